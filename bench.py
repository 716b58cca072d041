#!/usr/bin/env python3
"""Benchmark: time to a converged CPHF solve (max_j ||b - (I+A)x||_2 < 1e-8) on one GB300.

A step is one full ``solve_dimless_cphf`` of the workload through libcphf.  The default
workload is ``rhf_nao1200``: RHF with RI-J/RI-K response, nao=1200, naux=4000, nocc=120,
360 right-hand sides (120 atoms), the size the headline metric is quoted on.  The timed arm is
the mixed-precision solve with the learned preconditioner (split-FP16 tensor-core operator
inside defect correction whose every correction residual, the final one included, is
recomputed with the FP64-accurate exact-slice operator inside the solve).

* ``value``: the solve with its inputs resident in HBM (CUDA events on the library stream).
* ``e2e``: per step, from pinned host buffers through the public API: the packed cderi upload
  (``set_cderi``), ``make_response_preparation`` (Z/O, the FP16 / BF16 planes of B) and the
  solve with the right-hand side in and U1 out.
* ``fp64_plain``: the plain FP64 GPU solve of the same system.  Measured in full where it fits
  the run (nrhs <= 180); at the larger sizes its operator-call count comes from a measured FP64
  solve of a column subset and its per-call cost from measured FP64 applications at two widths
  (the K term is linear in the column count), labelled ``extrapolated``.
* Accuracy: U1 and the Hessian blocks of the mixed solve against the FP64 solve (all columns
  where the FP64 solve is measured in full, else the subset's columns and the Hessian blocks
  of the subset's atoms), and the native FP64 residual of the mixed solution.

``--impl reference`` times the reference algorithm on the host CPU instead (the numpy port in
``oracle/``, all cores), on bounded samples of the same workload, extrapolated and labelled.
``--apply-only`` times single operator applications (launch lists and profiler captures).

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
    "rhf_nao1200": "RHF CPHF, RI-JK response: nao=1200 naux=4000 nocc=120 nvir=1080 nrhs=360 (120 atoms)",
    "rhf_nao600": "RHF CPHF, RI-JK response: nao=600 naux=2000 nocc=60 nvir=540 nrhs=180 (60 atoms)",
    "rhf_nao24": "RHF CPHF, RI-JK response: nao=24 naux=84 nocc=5 nrhs=12 (4 atoms)",
    "rhf_nao300": "RHF CPHF, RI-JK response: nao=300 naux=1000 nocc=30 nrhs=90 (30 atoms)",
    "rhf_nao384_occ120": "RHF CPHF, RI-JK response: nao=384 naux=1280 nocc=120 nrhs=36 (12 atoms)",
    "rks_nao600": "RKS CPKS, RI-JK + LDA XC response on ~660k grid points: nao=600 naux=2000 nocc=60 nrhs=180",
    "uks_nao800": "UKS CPKS, RI-JK + LDA XC: nao=800 naux=2700 nocc=80/78 nrhs=240",
}
FULL_FP64_MAX_NRHS = 180   # above this the plain FP64 solve is extrapolated (config 4: ~2900 s)


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["cphf", "reference"], default="cphf")
    p.add_argument("--workload", default="rhf_nao1200")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 leg")
    p.add_argument("--fp64-full", action="store_true", help="always run the plain FP64 solve in full")
    p.add_argument("--fp64-cols", type=int, default=6,
                   help="columns of the measured FP64 subset solve (when the full solve is extrapolated)")
    p.add_argument("--fp64-app-cols", type=int, default=36,
                   help="width of the wider measured FP64 application (extrapolation, residual check)")
    p.add_argument("--e2e-steps", type=int, default=2, help="end-to-end steps (0: as many as --steps)")
    p.add_argument("--cpu-sample", type=int, default=0, help="RHS columns of the CPU baseline sample (0: auto)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg (profiling runs)")
    p.add_argument("--inner-tol", type=float, default=None, help="Krylov tol of the inner solves (library default)")
    p.add_argument("--no-graphs", action="store_true", help="run the inner operator eagerly (no CUDA graphs)")
    p.add_argument("--no-learned", action="store_true", help="do not use the trained network")
    p.add_argument("--learned-mode", type=int, default=1, choices=[1, 2],
                   help="1: learned preconditioner; 2: preconditioner and initial guess")
    p.add_argument("--no-learned-gain", action="store_true", help="skip the solve without the network")
    p.add_argument("--fp64-tol", type=float, default=1e-10, help="Krylov tol of the plain FP64 solve")
    p.add_argument("--fp64-lindep", type=float, default=1e-20,
                   help="Krylov lindep of the plain FP64 solve; the convergence test is max(lindep, tol^2), "
                        "so the default 1e-14 would stop it above the ||r|| < 1e-8 target")
    p.add_argument("--residual", type=int, default=2, choices=[0, 1, 2],
                   help="mixed solve's correction residuals: 0 FP64, 1 double-float, 2 double-float + "
                        "tensor-core K term and XC with exact BF16 slices")
    p.add_argument("--verify", type=int, default=2, choices=[0, 1, 2],
                   help="mixed solve's final check: 2 recomputed with the --residual operator, 1 native FP64, "
                        "0 updated with the split-precision operator")
    p.add_argument("--apply-only", action="store_true",
                   help="only time --reps operator applications of --nb columns (launch lists / captures)")
    p.add_argument("--nb", type=int, default=0, help="--apply-only: columns per application (0: all RHS)")
    p.add_argument("--reps", type=int, default=3, help="--apply-only: applications")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "accurate"],
                   help="--apply-only: operator (accurate: the mixed context's FP64-accurate operator, run by "
                        "finalize_cphf on all 3 natm perturbations)")
    return p.parse_args(argv)


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


def cpu_sample_cols(s, requested):
    """RHS columns of one bounded CPU operator sample (about 10-30 s on 16 cores)."""
    if requested > 0:
        return requested
    return 6 if s.nao <= 300 else (2 if s.nao <= 800 else 1)


def cpu_oracle_calibrate(s, ncols, wide_cols=0, calls=None):
    """Reference algorithm on the host (oracle port): the per-call cost model t0 + t1*nb from
    single operator applications at ncols and 2*ncols columns (and, if wide_cols > 0, one wider
    application that checks the model); the operator-call count from a real Krylov solve of
    ncols columns with the full-size operator, unless `calls` (measured elsewhere) is given."""
    drv = cpu_oracle_driver(s)
    nrhs, cut = _rhs_cut(s)
    x1, x2 = cut(ncols), cut(2 * ncols)
    t = time.perf_counter(); drv.response_dimless_cphf(x1); t1 = time.perf_counter() - t
    t = time.perf_counter(); drv.response_dimless_cphf(x2); t2 = time.perf_counter() - t
    slope = max((t2 - t1) / ncols, 1e-12)
    cal = dict(drv=drv, nrhs=nrhs, cut=cut, ncols=ncols, t1=t1, t2=t2, slope=slope, t_solve=None,
               calls=calls, calls_source="given", wide=None)
    if wide_cols > 0:
        t = time.perf_counter(); drv.response_dimless_cphf(cut(wide_cols)); tw = time.perf_counter() - t
        cal["wide"] = (wide_cols, tw, max(t1 - slope * ncols, 0.0) + slope * wide_cols)
    if calls is None:
        t = time.perf_counter()
        drv.solve_dimless_cphf(x1)
        cal["t_solve"] = time.perf_counter() - t
        cal["calls"] = drv.krylov_stats["aop_calls"]
        cal["calls_source"] = f"oracle solve of {ncols} columns"
    return cal


def cpu_oracle_value(cal, t_ncols):
    """Extrapolated solve time: calls x (t0 + t1 * nrhs), t0 from an application at ncols."""
    base = max(t_ncols - cal["slope"] * cal["ncols"], 0.0)
    return cal["calls"] * (base + cal["slope"] * cal["nrhs"])


def cpu_oracle_record(cal, value):
    cores = os.cpu_count()
    n, nrhs = cal["ncols"], cal["nrhs"]
    wide = ""
    if cal["wide"]:
        w, tw, pred = cal["wide"]
        wide = f"; check: {w}-column application measured {tw:.1f} s vs model {pred:.1f} s"
    solve = f", {cal['t_solve']:.1f} s" if cal["t_solve"] is not None else ""
    return dict(value=value, unit="s", cores=cores, kind="port", extrapolated=True,
                sample=(f"oracle (numpy/OpenBLAS, {cores} threads): operator applications at {n} and {2 * n} of "
                        f"{nrhs} RHS columns ({cal['t1']:.2f} s, {cal['t2']:.2f} s) give t0 + t1*nb; "
                        f"{cal['calls']} operator calls ({cal['calls_source']}{solve}); value = calls x "
                        f"(t0 + t1*{nrhs}), extrapolated{wide}"),
                calls=cal["calls"], matvec_s_per_col=cal["slope"])


def run_reference(args, world, rank):
    """The reference algorithm on the host cores.  The cost model and call count are calibrated
    once; every warm-up and timed step is one operator application of the oracle on the sample
    columns (a bounded sample of the solve), extrapolated to the full solve (labelled)."""
    if rank != 0:
        return
    from cphf_gb300 import synth
    s = synth.make_system(args.workload, seed=args.seed)
    ncols = cpu_sample_cols(s, args.cpu_sample)
    wide = 12 if s.nao >= 800 else 3 * s.natm
    cal = cpu_oracle_calibrate(s, ncols, wide_cols=wide)
    x = cal["cut"](cal["ncols"])
    values, walls = [], []
    for _ in range(args.warmup + args.steps):
        t = time.perf_counter()
        cal["drv"].response_dimless_cphf(x)
        walls.append(time.perf_counter() - t)
        values.append(cpu_oracle_value(cal, walls[-1]))
    value = statistics.median(values[args.warmup:])
    cb = cpu_oracle_record(cal, value)
    line = dict(metric=METRIC, value=value, unit="s", n_gpus=args.gpus, steps=args.steps, warmup=args.warmup,
                ms_per_step=value * 1e3, higher_is_better=False, scaling="weak", vs_baseline=None, dtype="f64",
                data=f"synthetic (seeded generator, {args.workload}, seed {args.seed})",
                config=dict(workload=args.workload, description=WORKLOAD_DESC.get(args.workload, args.workload)),
                impl="reference", extrapolated=True,
                measured_step_s=statistics.median(walls[args.warmup:]),
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
        return (d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0),
                d.get("bf16_tflops_sustained", d.get("bf16_tflops", 1700.0)), "measured")
    return 6800.0, 1900.0, 1700.0, "fallback"


def fcol(t):
    """col-major [nmo, nocc, 3, natm] view of a torch tensor stored with reversed C-order dims."""
    return t.permute(*reversed(range(t.dim())))


def f_to_torch(a, pin=False, device=None):
    """A Fortran-ordered numpy array as an F-contiguous torch view (pinned host or device)."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose(tuple(reversed(range(a.ndim))))))
    if pin:
        t = t.pin_memory()
    if device is not None:
        t = t.to(device)
    return fcol(t)


def cols_of(a, k):
    """The first k perturbation columns of [nmo, nocc, 3, natm] (or [nmo, nocc, ncol]) as [nmo, nocc, k]."""
    return np.asfortranarray(a.reshape(a.shape[0], a.shape[1], -1, order="F")[:, :, :k])


def with_cols(full, part, k):
    """A copy of `full` [n1, n2, 3, natm] whose first k perturbation columns are `part`'s."""
    out = np.array(full, order="F", copy=True)
    flat = out.reshape(out.shape[0], out.shape[1], -1, order="F")
    assert np.shares_memory(flat, out)
    flat[:, :, :k] = np.asarray(part).reshape(out.shape[0], out.shape[1], k, order="F")
    return out


def setup_ctx(cphf_gb300, s, precision, local, cderi=None, **cfg):
    ctx = cphf_gb300.Context(precision=precision, device=local, **cfg)
    prepare_ctx(ctx, s, cderi)
    return ctx


def prepare_ctx(ctx, s, cderi=None, mo=None):
    """set_cderi (+ grid) and make_response_preparation from the given (host or pinned) arrays."""
    ctx.set_cderi(s.cderi if cderi is None else cderi, s.scale_j, s.scale_k, nao=s.nao)
    if s.grid is not None:
        ctx.set_grid(s.grid.ao, s.grid.weights, s.grid.fxc, s.nspin, s.grid.atom_offsets)
    C, occ, e = mo if mo is not None else (s.mo_coeff, s.mo_occ, s.mo_energy)
    if s.nspin == 1:
        ctx.make_response_preparation(C[0], occ[0], e[0])
    else:
        ctx.make_response_preparation(C, occ, e)


def run_apply_only(args, local):
    """Time single operator applications (for launch lists and profiler captures)."""
    import cphf_gb300
    from cphf_gb300 import synth
    cphf_gb300.build()
    s = synth.make_system(args.workload, seed=args.seed)
    accurate = args.precision == "accurate"
    nb = 3 * s.natm if accurate else (args.nb or 3 * s.natm)
    ctx = setup_ctx(cphf_gb300, s, "mixed" if accurate else args.precision, local)
    rng = np.random.default_rng(args.seed + 1)
    mo1 = [rng.standard_normal((s.nao, s.nocc[t], nb)) for t in range(s.nspin)]
    mo1 = mo1 if s.nspin == 2 else mo1[0]
    op = ctx.response_dimless_cphf_lowp if args.precision == "mixed" else ctx.response_dimless_cphf
    if accurate:
        # the split-precision state first (its planes of B feed the exact slices' preparation),
        # then finalize_cphf, whose response is the FP64-accurate operator on mo1
        ctx.response_dimless_cphf_lowp(mo1)
        shp = [(s.nao, s.nocc[t], 3, s.natm) for t in range(s.nspin)]
        f1 = [rng.standard_normal(sh) for sh in shp]
        s1 = [rng.standard_normal(sh) for sh in shp]
        m1 = [m.reshape(sh, order="F") for m, sh in zip(mo1 if s.nspin == 2 else [mo1], shp)]
        if s.nspin == 1:
            f1, s1, m1 = f1[0], s1[0], m1[0]
        op = lambda _: ctx.finalize_cphf(f1, s1, m1)  # noqa: E731
    for r in range(args.reps):
        t0 = time.perf_counter()
        op(mo1)
        print(f"application {r}: {time.perf_counter() - t0:.4f} s ({args.workload}, nb={nb}, {args.precision})",
              flush=True)


def run_gpu(args, world, rank, local):
    import torch
    import cphf_gb300
    from cphf_gb300 import synth

    t_run0 = time.perf_counter()
    torch.cuda.set_device(local)
    cphf_gb300.build()
    t = time.perf_counter()
    s = synth.make_system(args.workload, seed=args.seed)
    synth_s = time.perf_counter() - t
    nspin = s.nspin
    nrhs = 3 * s.natm
    rhs_h = s.rhs if nspin == 2 else [s.rhs[0]]
    arg = (lambda v: v if nspin == 2 else v[0])
    dev = torch.device("cuda", local)

    weights = ROOT / "rstsr-showcase-hessian_gb300" / "cphf_gb300" / "mlp_weights.npy"
    learned = weights.exists() and not args.no_learned
    inner = {} if args.inner_tol is None else dict(inner_tol=args.inner_tol)
    mixed_cfg = dict(verify_residual=args.verify, use_learned_guess=args.learned_mode if learned else 0,
                     residual_dfloat=args.residual, cuda_graphs=0 if args.no_graphs else 1, **inner)
    torch.cuda.synchronize()
    t = time.perf_counter()
    mixed = setup_ctx(cphf_gb300, s, "mixed", local, **mixed_cfg)
    if learned:
        mixed.set_mlp_weights(np.load(weights))
    mixed.synchronize()
    setup_resident_s = time.perf_counter() - t

    # device-resident inputs and outputs (F-contiguous views of C-ordered tensors)
    rhs_d = [f_to_torch(r, device=dev) for r in rhs_h]
    out_d = [fcol(torch.empty(tuple(reversed(r.shape)), dtype=torch.float64, device=dev)) for r in rhs_h]
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
    x_mixed = [np.asfortranarray(o.cpu().numpy()) for o in out_d]

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

    # what the trained network gains: the same solve without it (same context, same box)
    gain = None
    if learned and not args.no_learned_gain:
        mixed.set_config(use_learned_guess=0)
        eg0, eg1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        eg0.record(stream)
        mixed.solve_dimless_cphf(arg(rhs_d), out=arg(out_d))
        eg1.record(stream)
        torch.cuda.synchronize()
        st0 = mixed.last_stats
        t_nolearn = eg0.elapsed_time(eg1) * 1e-3
        gain = dict(with_s=t_step, without_s=t_nolearn, gain=(t_nolearn - t_step) / t_nolearn,
                    mode=args.learned_mode,
                    lowp_columns_with=stats[-1]["lowp_matvec_columns"], lowp_columns_without=st0["lowp_matvec_columns"],
                    cycles_with=stats[-1]["cycles"], cycles_without=st0["cycles"])
        mixed.set_config(use_learned_guess=args.learned_mode)

    # end to end through the public API with pinned host buffers: per step the packed cderi
    # upload, the preparation (Z/O, B planes) and the solve (rhs in, U1 out)
    cderi_p = f_to_torch(s.cderi, pin=True)
    mo_p = ([f_to_torch(c, pin=True) for c in s.mo_coeff[:nspin]], [np.asarray(o) for o in s.mo_occ[:nspin]],
            [np.asarray(e) for e in s.mo_energy[:nspin]])
    rhs_p = [f_to_torch(r, pin=True) for r in rhs_h]
    out_p = [fcol(torch.empty(tuple(reversed(r.shape)), dtype=torch.float64).pin_memory()) for r in rhs_h]
    del rhs_d, out_d
    n_e2e = args.steps if args.e2e_steps <= 0 else min(args.e2e_steps, args.steps)
    h2d = (s.cderi.nbytes + sum(c.nbytes for c in s.mo_coeff[:nspin]) + sum(r.nbytes for r in rhs_h)
           + (s.grid.ao.nbytes + s.grid.weights.nbytes + s.grid.fxc.nbytes if s.grid is not None else 0))
    d2h = sum(r.nbytes for r in rhs_h)
    e2e_times, setup_times = [], []
    for _ in range(n_e2e):
        torch.cuda.synchronize()
        t = time.perf_counter()
        prepare_ctx(mixed, s, cderi=cderi_p, mo=mo_p)
        mixed.synchronize()
        setup_times.append(time.perf_counter() - t)
        mixed.solve_dimless_cphf(arg(rhs_p), out=arg(out_p))
        e2e_times.append(time.perf_counter() - t)
    t_e2e = max_over_ranks(world, statistics.median(e2e_times))
    setup_s = statistics.median(setup_times)
    x_e2e = [np.asfortranarray(o.numpy()) for o in out_p]
    e2e_same = max(float(np.abs(a - b).max()) for a, b in zip(x_e2e, x_mixed))
    tc_active = mixed.tensor_cores_active

    # finalize_cphf of the mixed solution on the mixed context (its response on the FP64-accurate
    # operator) and the Hessian, for the accuracy comparison below
    f1 = s.f1mo if nspin == 2 else s.f1mo[0]
    s1 = s.s1mo if nspin == 2 else s.s1mo[0]
    t = time.perf_counter()
    m1_mx, me_mx = mixed.finalize_cphf(f1, s1, arg(x_mixed))
    de_mx = mixed.get_cphf_hess(f1, s1, m1_mx, me_mx)
    finalize_s = time.perf_counter() - t
    m1_mx = m1_mx if nspin == 2 else [m1_mx]
    me_mx = me_mx if nspin == 2 else [me_mx]
    mixed.close()  # release its device memory before the FP64 context is built
    del cderi_p
    torch.cuda.empty_cache()

    # ---- plain FP64 GPU solve (the reference's arithmetic) and the accuracy of the mixed solve
    fp64 = setup_ctx(cphf_gb300, s, "fp64", local, cphf_tol=args.fp64_tol, cphf_lindep=args.fp64_lindep)
    fp64_line, accuracy = None, {}

    def residual_cols(x, k):
        """native FP64 max_j ||b_j - (I+A)x_j||_2 over the first k columns, and the application time"""
        bs = [cols_of(b, k) for b in rhs_h]
        xs = [cols_of(v, k) for v in x]
        fp64.synchronize()
        t0 = time.perf_counter()
        y = fp64.response_dimless_cphf(arg(xs))
        t_app = time.perf_counter() - t0
        y = y if nspin == 2 else [y]
        r = max(float(np.linalg.norm((b - v - w).reshape(-1, k, order="F"), axis=0).max())
                for b, v, w in zip(bs, xs, y))
        return r, t_app

    if not args.no_fp64:
        full = args.fp64_full or nrhs <= FULL_FP64_MAX_NRHS
        if full:
            t = time.perf_counter()
            x64 = fp64.solve_dimless_cphf(arg(rhs_h))
            t_fp64 = time.perf_counter() - t
            st64 = fp64.last_stats
            x64 = x64 if nspin == 2 else [x64]
            res_mixed, t_app = residual_cols(x_mixed, nrhs)
            res_64, _ = residual_cols(x64, nrhs)
            m1_64, me_64 = fp64.finalize_cphf(f1, s1, arg(x64))
            de_64 = fp64.get_cphf_hess(f1, s1, m1_64, me_64)
            m1_64 = m1_64 if nspin == 2 else [m1_64]
            accuracy = dict(columns=nrhs, atoms="all",
                            u1_max_abs_diff=max(float(np.abs(a - b).max()) for a, b in zip(m1_mx, m1_64)),
                            hessian_max_abs_diff=float(np.abs(de_mx - de_64).max()),
                            mixed_residual_fp64=res_mixed, fp64_residual_fp64=res_64)
            fp64_line = dict(value=t_fp64, unit="s", measured=True, aop_calls=st64["aop_calls"],
                             aop_columns=st64["aop_columns"], cycles=st64["cycles"], tol=args.fp64_tol,
                             lindep=args.fp64_lindep, application_s=t_app, application_cols=nrhs)
        else:
            # FP64 solve of the first k perturbation columns (the columns are independent
            # systems): call count, and U1 / Hessian reference for those columns
            k = args.fp64_cols
            k = max(3, (k // 3) * 3)  # whole atoms
            t = time.perf_counter()
            x64 = fp64.solve_dimless_cphf(arg([cols_of(r, k) for r in rhs_h]))
            t_sub = time.perf_counter() - t
            st64 = fp64.last_stats
            x64 = x64 if nspin == 2 else [x64]
            # FP64 applications at k and at a wider width: cost model t0 + t1 nb; the wider one is
            # also the native FP64 residual of the mixed solution on those columns
            res_mixed_k, t_k = residual_cols(x_mixed, k)
            w = min(args.fp64_app_cols, nrhs)
            res_mixed_w, t_w = residual_cols(x_mixed, w)
            t1 = (t_w - t_k) / max(w - k, 1)
            t0 = max(t_k - t1 * k, 0.0)
            per_call_full = t0 + t1 * nrhs
            res_64, _ = residual_cols(x64, k)
            # finalize of the subset columns in FP64; Hessian blocks of the subset's atoms from the
            # mixed finalize with those columns replaced (every block of atoms 0..k/3-1)
            natm_k = k // 3
            f1k = [cols_of(v, k).reshape(v.shape[0], v.shape[1], 3, natm_k, order="F") for v in
                   (s.f1mo[:nspin])]
            s1k = [cols_of(v, k).reshape(v.shape[0], v.shape[1], 3, natm_k, order="F") for v in
                   (s.s1mo[:nspin])]
            x64k = [v.reshape(v.shape[0], v.shape[1], 3, natm_k, order="F") for v in x64]
            m1k, mek = fp64.finalize_cphf(arg(f1k), arg(s1k), arg(x64k))
            m1k = m1k if nspin == 2 else [m1k]
            mek = mek if nspin == 2 else [mek]
            hyb_m1 = [with_cols(a, b, k) for a, b in zip(m1_mx, m1k)]
            hyb_me = [with_cols(a, b, k) for a, b in zip(me_mx, mek)]
            de_hyb = fp64.get_cphf_hess(f1, s1, arg(hyb_m1), arg(hyb_me))
            accuracy = dict(columns=k, atoms=f"0..{natm_k - 1} (every Hessian block with one of them)",
                            u1_max_abs_diff=max(float(np.abs(cols_of(a, k) - cols_of(b, k)).max())
                                                for a, b in zip(m1_mx, m1k)),
                            hessian_max_abs_diff=float(np.abs(de_mx - de_hyb).max()),
                            mixed_residual_fp64=max(res_mixed_k, res_mixed_w), mixed_residual_columns=w,
                            fp64_residual_fp64=res_64)
            fp64_line = dict(value=st64["aop_calls"] * per_call_full, unit="s", measured=False, extrapolated=True,
                             aop_calls=st64["aop_calls"], cycles=st64["cycles"], tol=args.fp64_tol,
                             lindep=args.fp64_lindep, subset_solve_s=t_sub, subset_columns=k,
                             application_s={str(k): t_k, str(w): t_w}, per_call_full_s=per_call_full,
                             how=(f"calls of a measured FP64 solve of {k} of {nrhs} columns x per-call time "
                                  f"t0 + t1*{nrhs} from measured FP64 applications at {k} and {w} columns"))
    fp64.close()

    # ---- roofline of the dominant kernel class in the timed region
    hbm, bf16, bf16_sus, peak_src = load_peaks()
    dom_name, dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    tensor_notes = {
        "kterm_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products",
        "tgen_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products",
        "wgen_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products",
        "term2_tcgen05_f16x3": "FP16 hi/lo, the tensor pipe executes 3 split products",
        "kterm_tcgen05_bf16x6_exact": "exact BF16 slices, the tensor pipe executes 21 slice products",
        "xc_tcgen05_f16x3": "per grid batch over its AO window, FP16 hi/lo, 3 split products",
        "xc_tcgen05_bf16x6_exact": "per grid batch over its AO window, exact BF16 slices, 21 slice products",
        "tgen_tcgen05_bf16x6_exact": "exact BF16 slices, the tensor pipe executes 21 slice products",
        "wgen_tcgen05_bf16x6_exact": "exact BF16 slices, the tensor pipe executes 21 slice products",
        "term2_tcgen05_bf16x6_exact": "exact BF16 slices, the tensor pipe executes 21 slice products",
        "kterm_tcgen05_bf16x4c_exact": "exact BF16 slices in correction precision, 10 slice products",
        "tgen_tcgen05_bf16x4c_exact": "exact BF16 slices in correction precision, 10 slice products",
        "wgen_tcgen05_bf16x4c_exact": "exact BF16 slices in correction precision, 10 slice products",
        "term2_tcgen05_bf16x4c_exact": "exact BF16 slices in correction precision, 10 slice products",
        "kterm_tcgen05_bf16x3c_exact": "exact BF16 slices in correction precision, 6 slice products",
        "tgen_tcgen05_bf16x3c_exact": "exact BF16 slices in correction precision, 6 slice products",
        "wgen_tcgen05_bf16x3c_exact": "exact BF16 slices in correction precision, 6 slice products",
        "term2_tcgen05_bf16x3c_exact": "exact BF16 slices in correction precision, 6 slice products",
        "xc_tcgen05_bf16c_exact": "per grid batch over its AO window, exact BF16 slices in correction precision "
                                  "(3 or 4 slices, 6 or 10 products)",
    }
    if dom_name in ("slice_scale_split", "slice_exact"):
        roof = dict(bound="hbm", achieved=dom["bytes"] / dom["ms"] / 1e6, peak=hbm, unit="GB/s",
                    peak_source=f"{peak_src} HBM copy; achieved counts the algorithmic bytes (operands read, "
                                "slice planes written) of the slicing / scaling kernels")
    elif dom_name == "gemm_fp64_simt":
        peak = measure_fp64_peak()
        roof = dict(bound="tensor", achieved=dom["flops"] / dom["ms"] / 1e9, peak=peak, unit="TFLOP/s",
                    peak_source="in-run cuBLAS FP64 GEMM 8192^3 (FP64 has no entry in MEASURED_PEAKS.json)")
    else:
        note = tensor_notes.get(dom_name, "")
        roof = dict(bound="tensor", achieved=dom["flops"] / dom["ms"] / 1e9, peak=bf16_sus, unit="TFLOP/s",
                    peak_source=(f"{peak_src} bf16 dense sustained (the kernel is timed inside a "
                                 f"{t_step:.0f} s solve; FP16 runs at the same rate; burst {bf16}); achieved "
                                 f"counts algorithmic FLOPs") + (f"; {note}" if note else ""))
    # DRAM bytes per launch: the ratio of ncu-measured DRAM bytes to the algorithmic bytes of
    # the same kernel on a small case (profiles/), times this run's algorithmic bytes per launch
    traffic_ratio = {"kterm_tcgen05_f16x3": 9.99 / 9.25,         # tc_term1_kernel, rhf_nao384_occ120
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
                "xc_tcgen05_f16x3": 3, "xc_tcgen05_bf16x6_exact": 21, "tgen_tcgen05_bf16x6_exact": 21,
                "wgen_tcgen05_bf16x6_exact": 21, "term2_tcgen05_bf16x6_exact": 21,
                "kterm_tcgen05_bf16x4c_exact": 10, "tgen_tcgen05_bf16x4c_exact": 10,
                "wgen_tcgen05_bf16x4c_exact": 10, "term2_tcgen05_bf16x4c_exact": 10,
                "kterm_tcgen05_bf16x3c_exact": 6, "tgen_tcgen05_bf16x3c_exact": 6,
                "wgen_tcgen05_bf16x3c_exact": 6, "term2_tcgen05_bf16x3c_exact": 6}.get(dom_name)
    if products and roof.get("peak"):
        roof.update(tensor_executed_tflops=roof["achieved"] * products,
                    tensor_executed_frac=roof["achieved"] * products / roof["peak"])
    roof.update(kernel=dom_name, frac=roof["achieved"] / roof["peak"] if roof.get("peak") else None, traffic=traffic,
                traffic_unit="bytes per launch" if traffic else None,
                launches=dom["launches"], avg_launch_ms=dom["ms"] / dom["launches"],
                share_of_step=dom["ms"] * 1e-3 / t_prof)

    cpu = None
    if rank == 0 and not args.no_cpu:
        ncols = cpu_sample_cols(s, args.cpu_sample)
        calls = fp64_line["aop_calls"] if (fp64_line and not fp64_line.get("measured")) else None
        cal = cpu_oracle_calibrate(s, ncols, calls=calls)
        if calls is not None:
            cal["calls_source"] = f"the GPU FP64 solve of {fp64_line['subset_columns']} columns (same algorithm)"
        cpu = cpu_oracle_record(cal, cpu_oracle_value(cal, cal["t1"]))

    st = stats[-1]
    line = dict(
        metric=METRIC, value=t_step, unit="s", n_gpus=args.gpus, steps=args.steps, warmup=args.warmup,
        ms_per_step=t_step * 1e3, higher_is_better=False, scaling="weak", vs_baseline=None,
        dtype=("f16x3 tensor-core operator / f32 / f64 defect correction"
               + {0: " (fp64 residuals)", 1: " (double-float residuals)",
                  2: " (residuals: bf16x6 exact-slice tensor-core K term and XC + double-float)"}[args.residual]),
        data=f"synthetic (seeded generator, {args.workload}, seed {args.seed})",
        config=dict(workload=args.workload, description=WORKLOAD_DESC.get(args.workload, args.workload),
                    precision="mixed", learned=(f"mode {args.learned_mode}" if learned else None),
                    residual_mode=args.residual, final_check=args.verify,
                    inner_tol=args.inner_tol if args.inner_tol is not None else 1e-6,
                    cuda_graphs=not args.no_graphs,
                    parallelism="replicas" if world > 1 else "single GPU",
                    l2="inputs larger than L2 (dense cderi FP64 %.1f GB)" % (s.nao ** 2 * s.naux * 8 / 1e9)),
        fp64_plain=fp64_line,
        speedup_vs_fp64_plain=None if fp64_line is None else fp64_line["value"] / t_step,
        speedup_e2e_vs_fp64_plain=None if fp64_line is None else fp64_line["value"] / t_e2e,
        accuracy=accuracy or None,
        solve_stats=dict(residual_max=st["residual_max"], residual_mode=st["residual_mode"],
                         refine_steps=st["refine_steps"], fp64_matvec_columns=st["fp64_matvec_columns"],
                         lowp_matvec_columns=st["lowp_matvec_columns"], cycles=st["cycles"],
                         tensor_cores=tc_active),
        learned_gain=gain,
        kernel_classes=dict(
            note="one profiled solve (eager operator, CUDA events per class) outside the timed region",
            solve_s=t_prof,
            **{k: dict(launches=v["launches"], ms=round(v["ms"], 3),
                       tflops=round(v["flops"] / max(v["ms"], 1e-9) / 1e9, 2),
                       gbs=round(v["bytes"] / max(v["ms"], 1e-9) / 1e6, 1)) for k, v in prof.items()}),
        e2e=dict(value=t_e2e, unit="s", h2d_bytes_per_step=int(h2d), d2h_bytes_per_step=int(d2h), steps=n_e2e,
                 setup_s=setup_s, solve_s=t_e2e - setup_s, same_answer_max_abs=e2e_same,
                 includes="packed cderi upload + make_response_preparation (Z/O, FP16 and BF16 planes of B) + "
                          "solve with rhs in and U1 out, pinned host buffers"),
        setup=dict(synth_s=synth_s, resident_setup_s=setup_resident_s, finalize_hessian_s=finalize_s),
        gpu_launches=int(launches),
        roofline=roof,
        cpu_baseline=None if cpu is None else {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        clocks=clk,
        wall_s=time.perf_counter() - t_run0,
    )
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.apply_only:
        run_apply_only(args, local)
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
