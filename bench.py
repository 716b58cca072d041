#!/usr/bin/env python3
"""Benchmark: time to a converged CPHF solve (max_j ||b - (I+A)x||_2 < 1e-8) on one GB300.

A step is one full ``solve_dimless_cphf`` of the workload (default ``rhf_nao600``:
nao=600, naux=2000, nocc=60, 180 right-hand sides, RHF with RI-J/RI-K response) through
libcphf.  The timed arm is the mixed-precision solve (split-FP16 tensor-core operator
inside FP64 defect correction); the plain FP64 GPU solve of the same system is timed once
beside it, and both solutions are verified with the FP64 operator outside the timed region.

``--impl reference`` times the reference algorithm on the host CPU instead (the numpy
port in ``oracle/``, all cores), on the same workload and metric.

Prints one JSON line (rank 0).  Multi-GPU runs are independent replicas (the path is not
sharded): one process per GPU via torchrun, max time over ranks.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "rstsr-showcase-hessian_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "time to converged CPHF (||r||<1e-8): mixed+learned vs plain FP64, same GB300"
WORKLOAD_DESC = {
    "rhf_nao600": "RHF CPHF, RI-JK response: nao=600 naux=2000 nocc=60 nvir=540 nrhs=180 (60 atoms)",
    "rhf_nao24": "RHF CPHF, RI-JK response: nao=24 naux=84 nocc=5 nrhs=12 (4 atoms)",
    "rhf_nao300": "RHF CPHF, RI-JK response: nao=300 naux=1000 nocc=30 nrhs=90 (30 atoms)",
    "rks_nao600": "RKS CPKS, RI-JK + LDA XC response on ~660k grid points: nao=600 naux=2000 nocc=60 nrhs=180",
    "uks_nao800": "UKS CPKS, RI-JK + LDA XC: nao=800 naux=2700 nocc=80/78 nrhs=240",
    "rhf_nao1200": "RHF CPHF, RI-JK response: nao=1200 naux=4000 nocc=120 nrhs=360",
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["cphf", "reference"], default="cphf")
    p.add_argument("--workload", default="rhf_nao600")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison solve")
    p.add_argument("--cpu-sample", type=int, default=6, help="RHS columns of the CPU baseline sample")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg (profiling runs)")
    p.add_argument("--inner-tol", type=float, default=None, help="Krylov tol of the inner solves (library default)")
    p.add_argument("--no-graphs", action="store_true", help="run the inner operator eagerly (no CUDA graphs)")
    p.add_argument("--verify-cols", type=int, default=0,
                   help="verify the FP64 residual on the first K perturbations only (0: all)")
    p.add_argument("--no-learned", action="store_true", help="do not use the trained initial guess")
    p.add_argument("--fp64-tol", type=float, default=1e-10, help="Krylov tol of the plain FP64 solve")
    p.add_argument("--fp64-lindep", type=float, default=1e-20,
                   help="Krylov lindep of the plain FP64 solve; the convergence test is max(lindep, tol^2), "
                        "so the default 1e-14 would stop it above the ||r|| < 1e-8 target")
    p.add_argument("--residual", type=int, default=2, choices=[0, 1, 2],
                   help="mixed solve's correction residual: 0 FP64, 1 double-float, 2 double-float + "
                        "tensor-core K term with exact BF16 slices")
    return p.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "cphf" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU (oracle) timing
def cpu_oracle_driver(s):
    """The reference algorithm restated on the CPU (oracle): RHF/UHF driver with the RI-JK and,
    for RKS/UKS workloads, the XC response plugins."""
    from oracle import cphf as ocphf
    from oracle import rijk as orijk
    from oracle import xc as oxc
    mocc = [s.mo_coeff[t][:, :s.nocc[t]] for t in range(s.nspin)]
    g = s.grid
    if s.nspin == 1:
        plugs = [lambda b: orijk.rhf_response_bra(s.cderi, s.mo_coeff[0], s.mo_occ[0], b, s.scale_j, s.scale_k)]
        if g is not None:
            plugs.append(lambda b: oxc.rks_response_bra(g.ao, g.weights, g.fxc, b, mocc[0]))
        return ocphf.RHF(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0], plugs, s.natm)
    plugs = [lambda b: orijk.uhf_response_bra(s.cderi, s.mo_coeff, s.mo_occ, b, s.scale_j, s.scale_k)]
    if g is not None:
        plugs.append(lambda b: oxc.uks_response_bra(g.ao, g.weights, g.fxc, b, mocc))
    return ocphf.UHF(s.mo_coeff, s.mo_occ, s.mo_energy, plugs, s.natm)


def _rhs_cut(s):
    nrhs = s.rhs[0].shape[2] * s.rhs[0].shape[3]
    rhs = [r.reshape(s.nao, s.nocc[t], nrhs, order="F") for t, r in enumerate(s.rhs[:s.nspin])]
    cut = (lambda k: rhs[0][:, :, :k]) if s.nspin == 1 else (lambda k: [r[:, :, :k] for r in rhs])
    return nrhs, cut


def cpu_oracle_calibrate(s, ncols):
    """Reference algorithm on the host (oracle port): a real Krylov solve of `ncols` RHS
    columns with the full-size operator gives the operator-call count; single matvecs at
    ncols and 2*ncols give the per-call cost model t0 + t1*nb."""
    drv = cpu_oracle_driver(s)
    nrhs, cut = _rhs_cut(s)
    x1, x2 = cut(ncols), cut(2 * ncols)
    t = time.perf_counter(); drv.response_dimless_cphf(x1); t1 = time.perf_counter() - t
    t = time.perf_counter(); drv.response_dimless_cphf(x2); t2 = time.perf_counter() - t
    slope = max((t2 - t1) / ncols, 1e-12)
    t = time.perf_counter()
    drv.solve_dimless_cphf(x1)
    t_solve = time.perf_counter() - t
    calls = drv.krylov_stats["aop_calls"]
    cols_per_call = drv.krylov_stats["aop_columns"] / max(calls, 1) / ncols
    return dict(drv=drv, nrhs=nrhs, cut=cut, ncols=ncols, t1=t1, t2=t2, slope=slope, t_solve=t_solve,
                calls=calls, cols_per_call=cols_per_call)


def cpu_oracle_value(cal, t_ncols):
    """Extrapolated solve time: calls x (t0 + t1 * nrhs * cols_per_call), t0 from a matvec at ncols."""
    base = max(t_ncols - cal["slope"] * cal["ncols"], 0.0)
    return cal["calls"] * (base + cal["slope"] * cal["nrhs"] * cal["cols_per_call"])


def cpu_oracle_record(cal, value):
    cores = os.cpu_count()
    n, nrhs = cal["ncols"], cal["nrhs"]
    return dict(value=value, unit="s", cores=cores, kind="port",
                sample=(f"oracle (numpy/OpenBLAS, {cores} threads) CPHF solve of {n} of {nrhs} RHS "
                        f"({cal['calls']} operator calls, {cal['t_solve']:.1f} s) plus matvecs at {n} and {2 * n} "
                        f"columns ({cal['t1']:.2f} s, {cal['t2']:.2f} s); value = calls x (t0 + t1*{nrhs}) "
                        f"extrapolated"),
                calls=cal["calls"], matvec_s_per_col=cal["slope"])


def cpu_oracle_estimate(s, ncols):
    """One calibration and its extrapolated solve time (the GPU arm's cpu_baseline)."""
    cal = cpu_oracle_calibrate(s, ncols)
    return cpu_oracle_record(cal, cpu_oracle_value(cal, cal["t1"]))


def run_reference(args, world, rank):
    """The reference algorithm on the host cores: the call count and per-column cost are
    calibrated once; every warm-up and timed step is one operator application of the oracle on
    the sample columns (a bounded sample of the solve), extrapolated to the full solve."""
    if rank != 0:
        return
    from cphf_gb300 import synth
    s = synth.make_system(args.workload, seed=args.seed)
    cal = cpu_oracle_calibrate(s, args.cpu_sample)
    x = cal["cut"](cal["ncols"])
    values = []
    for _ in range(args.warmup + args.steps):
        t = time.perf_counter()
        cal["drv"].response_dimless_cphf(x)
        values.append(cpu_oracle_value(cal, time.perf_counter() - t))
    value = statistics.median(values[args.warmup:])
    cb = cpu_oracle_record(cal, value)
    line = dict(metric=METRIC, value=value, unit="s", n_gpus=args.gpus, steps=args.steps, warmup=args.warmup,
                ms_per_step=value * 1e3, higher_is_better=False, scaling="weak", vs_baseline=None, dtype="f64",
                data=f"synthetic (seeded generator, {args.workload}, seed {args.seed})",
                config=dict(workload=args.workload, description=WORKLOAD_DESC.get(args.workload, args.workload)),
                impl="reference",
                cpu_baseline={k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                e2e=dict(value=value, unit="s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["nvidia-smi unavailable"])
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], None, set()
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=mx, reasons=sorted(reasons),
                    samples=len(sm))


def measure_fp64_peak():
    """cuBLAS FP64 GEMM rate on this GPU (torch.matmul), the denominator for FP64-pipe kernels."""
    import torch
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float64)
    b = torch.randn(n, n, device="cuda", dtype=torch.float64)
    a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(); a @ b; e1.record(); torch.cuda.synchronize()
    return 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def fcol(t):
    """col-major [nmo, nocc, 3, natm] view of a torch tensor stored with reversed C-order dims."""
    return t.permute(*reversed(range(t.dim())))


def run_gpu(args, world, rank, local):
    import torch
    import cphf_gb300
    from cphf_gb300 import synth

    torch.cuda.set_device(local)
    cphf_gb300.build()
    s = synth.make_system(args.workload, seed=args.seed)
    nspin = s.nspin
    rhs_h = s.rhs if nspin == 2 else [s.rhs[0]]

    def make_ctx(precision, **cfg):
        ctx = cphf_gb300.Context(precision=precision, device=local, **cfg)
        ctx.set_cderi(s.cderi, s.scale_j, s.scale_k)
        if s.grid is not None:
            ctx.set_grid(s.grid.ao, s.grid.weights, s.grid.fxc, nspin, s.grid.atom_offsets)
        if nspin == 1:
            ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])
        else:
            ctx.make_response_preparation(s.mo_coeff, s.mo_occ, s.mo_energy)
        return ctx

    weights = ROOT / "rstsr-showcase-hessian_gb300" / "cphf_gb300" / "mlp_weights.npy"
    learned = weights.exists() and not args.no_learned and nspin == 1
    inner = {} if args.inner_tol is None else dict(inner_tol=args.inner_tol)
    mixed = make_ctx("mixed", verify_residual=0, use_learned_guess=1 if learned else 0,
                     residual_dfloat=args.residual, cuda_graphs=0 if args.no_graphs else 1, **inner)
    if learned:
        mixed.set_mlp_weights(np.load(weights))
    # device-resident inputs and outputs (F-contiguous views of C-ordered tensors)
    rhs_d = [fcol(torch.from_numpy(np.ascontiguousarray(r.transpose(3, 2, 1, 0))).cuda()) for r in rhs_h]
    out_d = [fcol(torch.empty(tuple(reversed(r.shape)), dtype=torch.float64, device="cuda")) for r in rhs_h]
    arg = (lambda v: v if nspin == 2 else v[0])
    stream = torch.cuda.ExternalStream(mixed.stream)

    for _ in range(args.warmup):
        mixed.solve_dimless_cphf(arg(rhs_d), out=arg(out_d))
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    l0 = mixed.kernel_launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stats = []
    for _ in range(args.steps):
        mixed.solve_dimless_cphf(arg(rhs_d), out=arg(out_d))
        stats.append(mixed.last_stats)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    launches = mixed.kernel_launches - l0
    clk = clocks.stop()
    t_step = ev0.elapsed_time(ev1) * 1e-3 / args.steps
    t_step = max_over_ranks(world, t_step)

    # per-kernel-class breakdown: one more solve with the CUDA-event profiler on (which runs the
    # operator eagerly instead of replaying its graphs), outside the timed region
    mixed.profile(True)
    ep0, ep1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ep0.record(stream)
    mixed.solve_dimless_cphf(arg(rhs_d), out=arg(out_d))
    ep1.record(stream)
    torch.cuda.synchronize()
    t_prof = ep0.elapsed_time(ep1) * 1e-3
    prof = mixed.profile_report()
    mixed.profile(False)

    # end to end through the C ABI with pinned host buffers (copies inside the timed region)
    rhs_p = [torch.from_numpy(np.ascontiguousarray(r.transpose(3, 2, 1, 0))).pin_memory() for r in rhs_h]
    out_p = [torch.empty(tuple(reversed(r.shape)), dtype=torch.float64).pin_memory() for r in rhs_h]
    rhs_pf = [fcol(t) for t in rhs_p]
    out_pf = [fcol(t) for t in out_p]
    h2d = sum(r.nbytes for r in rhs_h)
    d2h = h2d
    t = time.perf_counter()
    for _ in range(args.steps):
        mixed.solve_dimless_cphf(arg(rhs_pf), out=arg(out_pf))
    t_e2e = max_over_ranks(world, (time.perf_counter() - t) / args.steps)
    x_mixed = [o.numpy().transpose(3, 2, 1, 0).copy(order="F") for o in out_p]
    tc_active = mixed.tensor_cores_active
    mixed.close()  # release its device memory before the FP64 context is built
    del rhs_d, out_d
    torch.cuda.empty_cache()

    # plain FP64 solve of the same system (the reference's arithmetic), timed once
    fp64 = make_ctx("fp64", cphf_tol=args.fp64_tol, cphf_lindep=args.fp64_lindep)
    fp64_res = None
    if not args.no_fp64:
        t = time.perf_counter()
        x64 = fp64.solve_dimless_cphf(arg(rhs_h))
        t_fp64 = time.perf_counter() - t
        st64 = fp64.last_stats
        x64 = x64 if nspin == 2 else [x64]

    # verification outside the timed regions: FP64 residuals (on the first --verify-cols
    # perturbations, all by default) and Hessian blocks
    ncols_v = args.verify_cols if args.verify_cols > 0 else None
    t_verify = [0.0]

    def residual(x):
        bs = [b.reshape(b.shape[0], b.shape[1], -1, order="F")[:, :, :ncols_v] for b in rhs_h]
        xs = [xx.reshape(xx.shape[0], xx.shape[1], -1, order="F")[:, :, :ncols_v] for xx in x]
        t = time.perf_counter()
        y = fp64.response_dimless_cphf(arg([np.asfortranarray(v) for v in xs]))
        t_verify[0] = time.perf_counter() - t
        y = y if nspin == 2 else [y]
        return max(float(np.linalg.norm((b - xx - yy).reshape(-1, b.shape[2], order="F"), axis=0).max())
                   for b, xx, yy in zip(bs, xs, y))

    res_mixed = residual(x_mixed)
    t_verify_mixed = t_verify[0]
    hess_diff = None
    if not args.no_fp64:
        fp64_res = residual(x64)
        f1 = s.f1mo if nspin == 2 else s.f1mo[0]
        s1 = s.s1mo if nspin == 2 else s.s1mo[0]
        h = []
        for x in (x_mixed, x64):
            m1, me = fp64.finalize_cphf(f1, s1, arg(x))
            h.append(fp64.get_cphf_hess(f1, s1, m1, me))
        hess_diff = float(np.abs(h[0] - h[1]).max())

    # roofline of the dominant kernel class in the timed region
    hbm, bf16, peak_src = load_peaks()
    dom_name, dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    tensor_notes = {
        "kterm_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products",
        "tgen_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products (twice: max, then planes)",
        "wgen_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products",
        "term2_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products",
        "kterm_tcgen05_bf16x6_exact": "exact BF16 slices, the tensor pipe executes 21 slice products",
        "xc_tcgen05_f16x3": "per grid batch over its AO window, FP16 hi/lo, 3 split products",
        "xc_tcgen05_bf16x6_exact": "per grid batch over its AO window, exact BF16 slices, 21 slice products",
    }
    if dom_name == "slice_scale_split":
        roof = dict(bound="hbm", achieved=dom["bytes"] / dom["ms"] / 1e6, peak=hbm, unit="GB/s",
                    peak_source=f"{peak_src} HBM copy; achieved counts the algorithmic bytes (operands read, "
                                "slice planes written) of the slicing / scaling kernels")
    elif dom_name == "gemm_fp64_simt":
        peak = measure_fp64_peak()
        roof = dict(bound="tensor", achieved=dom["flops"] / dom["ms"] / 1e9, peak=peak, unit="TFLOP/s",
                    peak_source="in-run cuBLAS FP64 GEMM 8192^3 (FP64 has no entry in MEASURED_PEAKS.json)")
    else:
        note = tensor_notes.get(dom_name, "")
        roof = dict(bound="tensor", achieved=dom["flops"] / dom["ms"] / 1e9, peak=bf16, unit="TFLOP/s",
                    peak_source=f"{peak_src} bf16 dense (FP16 runs at the same rate); achieved counts algorithmic "
                                f"FLOPs" + (f"; {note}" if note else ""))
    # DRAM bytes per launch: the ratio of ncu-measured DRAM bytes to the algorithmic bytes of
    # the same kernel on a small case (profiles/), times this run's algorithmic bytes per launch
    traffic_ratio = {"kterm_tcgen05_f16x3": 1.262 / 1.18,        # tc_term1_kernel, rhf_nao300
                     "kterm_tcgen05_bf16x6_exact": 5.954 / 5.22}  # tc_slice_kernel<Exact6>, rhf_nao300
    traffic = None
    if dom_name in traffic_ratio and dom.get("bytes", 0) > 0:
        traffic = traffic_ratio[dom_name] * dom["bytes"] / dom["launches"]
    if dom_name.startswith("xc_grouped"):
        roof.update(bound="fp64 pipe" if dom_name.endswith("fp64") else "fp32 pipe", peak=None,
                    peak_source="SIMT GEMM (no tensor-core form); see the per-class TFLOP/s")
    # products the tensor pipe executes per algorithmic FLOP (slices x slices kept)
    products = {"kterm_tcgen05_f16x3": 3, "tgen_tcgen05_f16x3": 3, "wgen_tcgen05_f16x3": 3,
                "term2_tcgen05_f16x3": 3, "kterm_tcgen05_bf16x6_exact": 21,
                "xc_tcgen05_f16x3": 3, "xc_tcgen05_bf16x6_exact": 21}.get(dom_name)
    if products and roof.get("peak"):
        roof.update(tensor_executed_tflops=roof["achieved"] * products,
                    tensor_executed_frac=roof["achieved"] * products / roof["peak"])
    roof.update(kernel=dom_name, frac=roof["achieved"] / roof["peak"] if roof.get("peak") else None, traffic=traffic,
                traffic_unit="bytes per launch" if traffic else None,
                launches=dom["launches"], avg_launch_ms=dom["ms"] / dom["launches"],
                share_of_step=dom["ms"] * 1e-3 / t_prof)

    cpu = cpu_oracle_estimate(s, args.cpu_sample) if rank == 0 and not args.no_cpu else None
    st = stats[-1]
    line = dict(
        metric=METRIC, value=t_step, unit="s", n_gpus=args.gpus, steps=args.steps, warmup=args.warmup,
        ms_per_step=t_step * 1e3, higher_is_better=False, scaling="weak", vs_baseline=None,
        dtype=("f16x3 tensor-core operator / f32 / f64 defect correction"
               + {0: " (fp64 residual)", 1: " (double-float residual)",
                  2: " (residual: bf16x6 exact-slice tensor-core K term and XC + double-float)"}[args.residual]),
        data=f"synthetic (seeded generator, {args.workload}, seed {args.seed})",
        config=dict(workload=args.workload, description=WORKLOAD_DESC.get(args.workload, args.workload),
                    precision="mixed", learned_guess=learned, residual_mode=args.residual,
                    inner_tol=args.inner_tol if args.inner_tol is not None else 1e-6,
                    cuda_graphs=not args.no_graphs,
                    parallelism="replicas" if world > 1 else "single GPU",
                    l2="inputs larger than L2 (dense cderi FP64 %.1f GB)" % (s.nao ** 2 * s.naux * 8 / 1e9)),
        fp64_plain=None if args.no_fp64 else dict(value=t_fp64, unit="s", aop_calls=st64["aop_calls"],
                                                  cycles=st64["cycles"], tol=args.fp64_tol,
                                                  lindep=args.fp64_lindep),
        speedup_vs_fp64_plain=None if args.no_fp64 else t_fp64 / t_step,
        residual=dict(mixed_verified=res_mixed, fp64_plain_verified=fp64_res, target=1e-8,
                      verified_columns=ncols_v or int(np.prod(rhs_h[0].shape[2:])),
                      fp64_operator_s=t_verify_mixed),
        hessian_max_abs_diff_vs_fp64=hess_diff,
        solve_stats=dict(refine_steps=st["refine_steps"], fp64_matvec_columns=st["fp64_matvec_columns"],
                         lowp_matvec_columns=st["lowp_matvec_columns"], cycles=st["cycles"],
                         tensor_cores=tc_active),
        kernel_classes=dict(
            note="one profiled solve (eager operator, CUDA events per class) outside the timed region",
            solve_s=t_prof,
            **{k: dict(launches=v["launches"], ms=round(v["ms"], 3),
                       tflops=round(v["flops"] / max(v["ms"], 1e-9) / 1e9, 2),
                       gbs=round(v["bytes"] / max(v["ms"], 1e-9) / 1e6, 1)) for k, v in prof.items()}),
        e2e=dict(value=t_e2e, unit="s", h2d_bytes_per_step=h2d, d2h_bytes_per_step=d2h),
        gpu_launches=int(launches),
        roofline=roof,
        cpu_baseline=None if cpu is None else {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        clocks=clk,
    )
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
