"""ctypes binding of libcphf (include/cphf.h) with the reference's call surface.

Method names follow the reference crate: ``make_response_preparation`` and
``get_response_bra`` of ``RHessElecInteractAPI`` (``src/hessian/trait_rhess.rs:162,189``; UHF ``trait_uhess.rs:152,171``),
``response_mo`` / ``response_dimless_cphf`` / ``solve_dimless_cphf`` /
``finalize_cphf`` / ``get_cphf_hess`` of ``RHessSCF`` / ``UHessSCF``
(``src/hessian/rscf.rs``, ``uscf.rs``) and ``krylov_block``
(``src/util/krylov_block.rs:39-47``).  Arrays are numpy (host) or torch (device)
float64 arrays with the reference's col-major meaning: numpy arrays are passed
Fortran-ordered; torch tensors must be F-contiguous views.  Where the reference
panics this raises :class:`CphfError` (:class:`KrylovNotConverged` for
``krylov_block.rs:188-194``).

Every computation runs in libcphf on the GPU; there is no CPU path here, and
loading fails loudly when the library has not been built.
"""

import ctypes
from pathlib import Path

import numpy as np

_LIB = None
LIB_PATH = Path(__file__).resolve().parent / "libcphf.so"

OK, ERR_SHAPE, ERR_NOT_CONVERGED, ERR_NONFINITE, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_STATE, ERR_ARG = range(9)
PRECISION = {"fp64": 0, "mixed": 1}

EXPORTS = [
    "cphf_config_default", "cphf_ctx_create", "cphf_ctx_destroy", "cphf_ctx_set_config",
    "cphf_status_string", "cphf_last_error", "cphf_ctx_stream", "cphf_ctx_synchronize",
    "cphf_ctx_device_bytes", "cphf_ctx_kernel_launches", "cphf_rijk_set_cderi", "cphf_xc_set_grid",
    "cphf_set_nao", "cphf_prepare", "cphf_response_bra", "cphf_plugin_response_bra",
    "cphf_response_mo", "cphf_response_dimless", "cphf_response_dimless_lowp", "cphf_solve_dimless_cphf",
    "cphf_finalize_cphf",
    "cphf_get_cphf_hess", "cphf_krylov_block", "cphf_dense_op_create", "cphf_dense_op_apply",
    "cphf_dense_op_destroy", "cphf_copy", "cphf_mlp_set_weights", "cphf_ctx_tensor_cores_active",
    "cphf_ctx_profile", "cphf_ctx_profile_report", "cphf_mlp_get_weights", "cphf_mlp_features",
    "cphf_mlp_forward", "cphf_mlp_loss_grad", "cphf_mlp_train", "cphf_rij_noalloc_capacity",
    "cphf_rij_response_bra_noalloc", "cphf_j2c_decompose", "cphf_rijk_set_j3c", "cphf_rijk_get_cderi",
    "cphf_compute_dimless_cphf_rhs", "cphf_xc_set_grid_ex",
]
MLP_NWEIGHTS = 4546


class ProfEntry(ctypes.Structure):
    _fields_ = [
        ("name", ctypes.c_char * 32),
        ("launches", ctypes.c_int64),
        ("ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
        ("flops", ctypes.c_double),
        ("bytes", ctypes.c_double),
    ]


class Config(ctypes.Structure):
    _fields_ = [
        ("level_shift", ctypes.c_double),
        ("cphf_tol", ctypes.c_double),
        ("cphf_max_cycle", ctypes.c_int64),
        ("cphf_max_space", ctypes.c_int64),
        ("cphf_lindep", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("residual_tol", ctypes.c_double),
        ("inner_tol", ctypes.c_double),
        ("max_refine", ctypes.c_int64),
        ("use_learned_guess", ctypes.c_int32),
        ("verbose", ctypes.c_int32),
        ("aux_chunk", ctypes.c_int64),
        ("tensor_cores", ctypes.c_int32),
        ("verify_residual", ctypes.c_int32),
        ("fp64_every_step", ctypes.c_int32),
        ("xc_chunk_points", ctypes.c_int64),
        ("residual_dfloat", ctypes.c_int32),
        ("cuda_graphs", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("aop_calls", ctypes.c_int64),
        ("aop_columns", ctypes.c_int64),
        ("cycles", ctypes.c_int64),
        ("restarts", ctypes.c_int64),
        ("max_innerprod", ctypes.c_double),
        ("residual_max", ctypes.c_double),
        ("fp64_matvec_columns", ctypes.c_int64),
        ("lowp_matvec_columns", ctypes.c_int64),
        ("refine_steps", ctypes.c_int64),
        ("seconds", ctypes.c_double),
        ("residual_mode", ctypes.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class J2cInfo(ctypes.Structure):
    _fields_ = [
        ("eig_fallback", ctypes.c_int32),
        ("jacobi_sweeps", ctypes.c_int32),
        ("min_diag", ctypes.c_double),
        ("seconds_decompose", ctypes.c_double),
        ("seconds_solve", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


AOP_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                          ctypes.c_void_p, ctypes.c_void_p)


class CphfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class KrylovNotConverged(CphfError):
    pass


def load_library():
    """Load libcphf.so (built by ``cphf_gb300._build.build``); raise if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is not built: run cphf_gb300._build.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(str(LIB_PATH))
    vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_double
    pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "cphf_config_default": ([ctypes.POINTER(Config)], i32),
        "cphf_ctx_create": ([ctypes.POINTER(Config), ctypes.POINTER(vp)], i32),
        "cphf_ctx_destroy": ([vp], i32),
        "cphf_ctx_set_config": ([vp, ctypes.POINTER(Config)], i32),
        "cphf_status_string": ([i32], ctypes.c_char_p),
        "cphf_last_error": ([vp], ctypes.c_char_p),
        "cphf_ctx_stream": ([vp], vp),
        "cphf_ctx_synchronize": ([vp], i32),
        "cphf_ctx_device_bytes": ([vp], i64),
        "cphf_ctx_kernel_launches": ([vp], i64),
        "cphf_rijk_set_cderi": ([vp, vp, i64, i64, dbl, dbl], i32),
        "cphf_xc_set_grid": ([vp, vp, vp, vp, i64, i32, vp, i64], i32),
        "cphf_set_nao": ([vp, i64], i32),
        "cphf_prepare": ([vp, i32, pp, pp, pp, i64], i32),
        "cphf_response_bra": ([vp, pp, i64, pp], i32),
        "cphf_plugin_response_bra": ([vp, i32, pp, i64, pp], i32),
        "cphf_response_mo": ([vp, pp, i64, pp], i32),
        "cphf_response_dimless": ([vp, pp, i64, pp], i32),
        "cphf_response_dimless_lowp": ([vp, pp, i64, pp], i32),
        "cphf_solve_dimless_cphf": ([vp, pp, i64, pp, pp, ctypes.POINTER(Stats)], i32),
        "cphf_finalize_cphf": ([vp, pp, pp, i64, pp, pp], i32),
        "cphf_get_cphf_hess": ([vp, pp, pp, pp, pp, i64, vp], i32),
        "cphf_krylov_block": ([vp, AOP_FN, vp, vp, vp, i64, i64, dbl, i64, i64, dbl, vp,
                               ctypes.POINTER(Stats)], i32),
        "cphf_dense_op_create": ([vp, vp, i64, ctypes.POINTER(vp)], i32),
        "cphf_dense_op_destroy": ([vp], i32),
        "cphf_copy": ([vp, vp, vp, i64], i32),
        "cphf_mlp_set_weights": ([vp, vp, i64], i32),
        "cphf_ctx_tensor_cores_active": ([vp], i32),
        "cphf_ctx_profile": ([vp, i32], i32),
        "cphf_ctx_profile_report": ([vp, ctypes.POINTER(ProfEntry), i32], i32),
        "cphf_mlp_get_weights": ([vp, vp, i64], i32),
        "cphf_mlp_features": ([vp, pp, i64, vp, i64, ctypes.POINTER(i64)], i32),
        "cphf_mlp_forward": ([vp, vp, i64, vp, i32], i32),
        "cphf_mlp_loss_grad": ([vp, vp, vp, i64, ctypes.POINTER(ctypes.c_float), vp], i32),
        "cphf_mlp_train": ([vp, vp, vp, i64, i64, i64, ctypes.c_float, ctypes.c_uint64, vp], i32),
        "cphf_j2c_decompose": ([vp, vp, i64, dbl, vp, ctypes.POINTER(J2cInfo)], i32),
        "cphf_rijk_set_j3c": ([vp, vp, vp, i64, i64, dbl, dbl, dbl, ctypes.POINTER(J2cInfo)], i32),
        "cphf_rijk_get_cderi": ([vp, vp], i32),
        "cphf_compute_dimless_cphf_rhs": ([vp, vp, pp, vp, i64, pp, pp, pp], i32),
        "cphf_xc_set_grid_ex": ([vp, i32, vp, i32, vp, vp, i64, i32, vp, i64], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    lib.cphf_dense_op_apply.restype = ctypes.c_int
    _LIB = lib
    return lib


def _is_torch(a):
    return type(a).__module__.startswith("torch")


class _Keep:
    """Holds converted arrays alive for the duration of a call and hands out pointers."""

    def __init__(self):
        self.refs = []

    def ptr(self, a):
        if a is None:
            return None
        if _is_torch(a):
            import torch
            if a.dtype != torch.float64:
                raise TypeError("torch arrays must be float64")
            if not _is_fcontig(a):
                raise ValueError("torch arrays must be F-contiguous (col-major) views")
            self.refs.append(a)
            return ctypes.c_void_p(a.data_ptr())
        arr = np.asfortranarray(a, dtype=np.float64)
        self.refs.append(arr)
        return ctypes.c_void_p(arr.ctypes.data)

    def ptrs(self, arrays):
        vals = [self.ptr(a) for a in arrays]
        arr = (ctypes.c_void_p * len(vals))(*[v.value if v is not None else None for v in vals])
        self.refs.append(arr)
        return ctypes.cast(arr, ctypes.POINTER(ctypes.c_void_p))


def _is_fcontig(t):
    expect = 1
    for size, stride in zip(t.shape, t.stride()):
        if size != 1 and stride != expect:
            return False
        expect *= size
    return True


def _shape(a):
    return tuple(a.shape) if hasattr(a, "shape") else np.shape(a)


def _nprop(shape):
    return int(np.prod(shape[2:])) if len(shape) > 2 else 1


class Context:
    """One libcphf context on one GPU (a set of plugins plus the CPHF driver state)."""

    def __init__(self, precision="fp64", device=0, **cfg):
        self.lib = load_library()
        self.cfg = Config()
        self.lib.cphf_config_default(ctypes.byref(self.cfg))
        self.cfg.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
        self.cfg.device = device
        for k, v in cfg.items():
            setattr(self.cfg, k, v)
        h = ctypes.c_void_p()
        self._check(self.lib.cphf_ctx_create(ctypes.byref(self.cfg), ctypes.byref(h)), ctx=False)
        self.h = h
        self.nspin = None
        self.nocc = None
        self.nmo = None
        self.nao = None
        self.last_stats = None

    # -- plumbing ------------------------------------------------------------------------
    def _check(self, status, ctx=True):
        if status == OK:
            return
        msg = self.lib.cphf_last_error(self.h).decode() if ctx else "context creation failed"
        if not msg:
            msg = self.lib.cphf_status_string(status).decode()
        if status == ERR_NOT_CONVERGED:
            raise KrylovNotConverged(status, msg)
        raise CphfError(status, msg)

    def close(self):
        if getattr(self, "h", None):
            self.lib.cphf_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_config(self, **cfg):
        for k, v in cfg.items():
            if k == "precision" and isinstance(v, str):
                v = PRECISION[v]
            setattr(self.cfg, k, v)
        self._check(self.lib.cphf_ctx_set_config(self.h, ctypes.byref(self.cfg)))

    @property
    def stream(self):
        return self.lib.cphf_ctx_stream(self.h)

    @property
    def device_bytes(self):
        return self.lib.cphf_ctx_device_bytes(self.h)

    @property
    def kernel_launches(self):
        return self.lib.cphf_ctx_kernel_launches(self.h)

    def synchronize(self):
        self._check(self.lib.cphf_ctx_synchronize(self.h))

    @property
    def tensor_cores_active(self):
        return bool(self.lib.cphf_ctx_tensor_cores_active(self.h))

    def profile(self, enable=True):
        """Start (clearing old records) or stop per-kernel-class CUDA-event timing."""
        self._check(self.lib.cphf_ctx_profile(self.h, 1 if enable else 0))

    def profile_report(self):
        """``{class: {launches, ms, max_ms, flops, bytes}}`` of the recorded launches."""
        buf = (ProfEntry * 32)()
        n = self.lib.cphf_ctx_profile_report(self.h, buf, 32)
        if n < 0:
            self._check(ERR_CUDA)
        return {buf[i].name.decode(): dict(launches=buf[i].launches, ms=buf[i].ms, max_ms=buf[i].max_ms,
                                           flops=buf[i].flops, bytes=buf[i].bytes) for i in range(n)}

    # -- plugins ---------------------------------------------------------------------------
    def set_cderi(self, cderi, scale_j=1.0, scale_k=1.0, nao=None):
        """``RHessRIJK::new_with_cderi`` (src/ri_jk/hess_r.rs:1774-1794); cderi ``[nao_tp, naux]``."""
        nao_tp, naux = cderi.shape
        if nao is None:
            nao = int(round((np.sqrt(8 * nao_tp + 1) - 1) / 2))
        if nao * (nao + 1) // 2 != nao_tp:
            raise CphfError(ERR_SHAPE, "cderi rows are not a packed triangle")
        k = _Keep()
        self._check(self.lib.cphf_rijk_set_cderi(self.h, k.ptr(cderi), nao, naux, scale_j, scale_k))
        self.nao = nao
        self.naux = naux

    def j2c_decompose(self, j2c, threshold=1e-14):
        """``decomp_j2c_cd(j2c, threshold, Upper)`` (src/ri_jk/pure_decompose.rs:29-57) on the GPU:
        returns ``(U, info)`` with ``j2c = U^T U``; ``threshold=None`` disables the fallback."""
        naux = j2c.shape[0]
        U = np.zeros((naux, naux), order="F")
        info = J2cInfo()
        k = _Keep()
        self._check(self.lib.cphf_j2c_decompose(self.h, k.ptr(j2c), naux, -1.0 if threshold is None else threshold,
                                                k.ptr(U), ctypes.byref(info)))
        return U, info.as_dict()

    def set_j3c(self, j3c, j2c, scale_j=1.0, scale_k=1.0, threshold=1e-14, nao=None):
        """``generate_cderi_with_decomp`` + ``new_with_cderi`` (src/ri_jk/hess_r.rs:1725-1735,
        1752): cderi = j3c U^-1 with j2c = U^T U, built on the GPU in FP64; returns the info dict."""
        nao_tp, naux = j3c.shape
        if nao is None:
            nao = int(round((np.sqrt(8 * nao_tp + 1) - 1) / 2))
        if nao * (nao + 1) // 2 != nao_tp:
            raise CphfError(ERR_SHAPE, "j3c rows are not a packed triangle")
        info = J2cInfo()
        k = _Keep()
        self._check(self.lib.cphf_rijk_set_j3c(self.h, k.ptr(j3c), k.ptr(j2c), nao, naux, scale_j, scale_k,
                                               -1.0 if threshold is None else threshold, ctypes.byref(info)))
        self.nao = nao
        self.naux = naux
        return info.as_dict()

    def get_cderi(self, out=None):
        """The RI-JK plugin's packed cderi ``[nao_tp, naux]`` (host array, or into ``out``)."""
        if out is None:
            if getattr(self, "naux", None) is None:
                raise CphfError(ERR_STATE, "RI-JK plugin not set")
            out = np.zeros((self.nao * (self.nao + 1) // 2, self.naux), order="F")
        k = _Keep()
        self._check(self.lib.cphf_rijk_get_cderi(self.h, k.ptr(out)))
        return out

    def set_nao(self, nao):
        self._check(self.lib.cphf_set_nao(self.h, nao))
        self.nao = nao

    def set_grid(self, ao, weights, fxc, nspin=1, batch_offsets=None):
        """XC plugin data: ``ao [ngrids, nao]``, ``weights [ngrids]``, ``fxc`` ``[ngrids]`` or ``[ngrids, 2, 2]``."""
        k = _Keep()
        ngrids = ao.shape[0]
        offs = None
        nb = 0
        if batch_offsets is not None:
            offs_arr = np.ascontiguousarray(batch_offsets, dtype=np.int64)
            k.refs.append(offs_arr)
            offs = ctypes.c_void_p(offs_arr.ctypes.data)
            nb = len(offs_arr) - 1
        self._check(self.lib.cphf_xc_set_grid(self.h, k.ptr(ao), k.ptr(weights), k.ptr(fxc), ngrids, nspin,
                                              offs, nb))

    def set_grid_ex(self, den_type, ao, weights, fxc_eff, nspin=1, batch_offsets=None):
        """XC plugin of any density type: ``den_type`` "rho" / "sigma" / "tau" (or 0 / 1 / 2),
        ``ao [ngrids, nao, ncomp]`` (value and first derivatives), ``fxc_eff [ngrids, nvar, nvar]``
        (RKS) or ``[ngrids, nvar, 2, nvar, 2]`` (UKS)."""
        den = {"rho": 0, "sigma": 1, "tau": 2}.get(den_type, den_type)
        k = _Keep()
        ao = np.asarray(ao) if not _is_torch(ao) else ao
        ngrids, ncomp = ao.shape[0], (ao.shape[2] if len(ao.shape) > 2 else 1)
        offs, nb = None, 0
        if batch_offsets is not None:
            offs_arr = np.ascontiguousarray(batch_offsets, dtype=np.int64)
            k.refs.append(offs_arr)
            offs = ctypes.c_void_p(offs_arr.ctypes.data)
            nb = len(offs_arr) - 1
        self._check(self.lib.cphf_xc_set_grid_ex(self.h, den, k.ptr(ao), ncomp, k.ptr(weights), k.ptr(fxc_eff),
                                                 ngrids, nspin, offs, nb))

    def make_response_preparation(self, mo_coeff, mo_occ, mo_energy):
        """``make_response_preparation`` plus orbital energies; RHF arrays or UHF two-spin lists."""
        uhf = isinstance(mo_coeff, (list, tuple))
        C = list(mo_coeff) if uhf else [mo_coeff]
        occ = list(mo_occ) if uhf else [mo_occ]
        e = list(mo_energy) if uhf else [mo_energy]
        k = _Keep()
        nmo = C[0].shape[1]
        self._check(self.lib.cphf_prepare(self.h, len(C), k.ptrs(C), k.ptrs(occ), k.ptrs(e), nmo))
        self.nspin = len(C)
        self.nocc = [int((np.asarray(o.cpu() if _is_torch(o) else o) > 0).sum()) for o in occ]
        self.nmo = nmo
        self.nao = C[0].shape[0]

    # -- responses -------------------------------------------------------------------------
    def _spins(self, x):
        if self.nspin is None:
            raise CphfError(ERR_STATE, "make_response_preparation has not been called")
        uhf = isinstance(x, (list, tuple))
        if uhf != (self.nspin == 2):
            raise CphfError(ERR_SHAPE, "spin structure of the argument does not match the preparation")
        return (list(x) if uhf else [x]), uhf

    def _call_spin(self, fn, x, out_rows, extra=()):
        xs, uhf = self._spins(x)
        shapes = [_shape(v) for v in xs]
        nprop = _nprop(shapes[0])
        outs = [np.zeros((out_rows(s),) + tuple(shapes[s][1:]), order="F") for s in range(len(xs))]
        k = _Keep()
        self._check(fn(self.h, *extra, k.ptrs(xs), nprop, k.ptrs(outs)))
        return outs if uhf else outs[0]

    def get_response_bra(self, bra, plugin=None):
        """``get_response_bra`` summed over the set plugins (or one: ``"rijk"`` / ``"xc"``)."""
        if plugin is None:
            return self._call_spin(self.lib.cphf_response_bra, bra, lambda s: self.nao)
        which = {"rijk": 0, "xc": 1}[plugin]
        return self._call_spin(self.lib.cphf_plugin_response_bra, bra, lambda s: self.nao, (which,))

    def response_mo(self, mo1):
        return self._call_spin(self.lib.cphf_response_mo, mo1, lambda s: self.nmo)

    def response_dimless_cphf(self, mo1):
        return self._call_spin(self.lib.cphf_response_dimless, mo1, lambda s: self.nmo)

    def response_dimless_cphf_lowp(self, mo1):
        """The dimensionless operator in the split-precision arithmetic of the mixed solve."""
        return self._call_spin(self.lib.cphf_response_dimless_lowp, mo1, lambda s: self.nmo)

    def solve_dimless_cphf(self, rhs, x0=None, out=None):
        """``solve_dimless_cphf``; statistics of the solve go to ``self.last_stats``."""
        xs, uhf = self._spins(rhs)
        nprop = _nprop(_shape(xs[0]))
        if out is None:
            out = [np.zeros(_shape(v), order="F") for v in xs]
        else:
            out = list(out) if uhf else [out]
        k = _Keep()
        st = Stats()
        x0p = None
        if x0 is not None:
            x0s, _ = self._spins(x0)
            x0p = k.ptrs(x0s)
        status = self.lib.cphf_solve_dimless_cphf(self.h, k.ptrs(xs), nprop, x0p, k.ptrs(out), ctypes.byref(st))
        self.last_stats = st.as_dict()
        self._check(status)
        return out if uhf else out[0]

    def compute_dimless_cphf_rhs(self, f1ao_core, f1bra_el, s1ao):
        """``compute_dimless_cphf_rhs`` (src/hessian/rscf.rs:104-182, uscf.rs:78-173): returns
        ``(rhs, f1mo, s1mo)`` (RHF arrays or UHF two-spin lists) from the skeleton derivatives
        ``f1ao_core`` / ``s1ao`` ``[nao, nao, 3, natm]`` and ``f1bra_el`` ``[nao, nocc_s, 3, natm]``
        (per spin for UHF; ``f1ao_core`` / ``f1bra_el`` may be None)."""
        if self.nspin is None:
            raise CphfError(ERR_STATE, "make_response_preparation has not been called")
        natm = int(np.prod(_shape(s1ao)[2:])) // 3
        tail = tuple(_shape(s1ao)[2:])
        el = None
        if f1bra_el is not None:
            el, _ = self._spins(f1bra_el)
        outs = [[np.zeros((self.nmo, self.nocc[s]) + tail, order="F") for s in range(self.nspin)] for _ in range(3)]
        k = _Keep()
        self._check(self.lib.cphf_compute_dimless_cphf_rhs(
            self.h, k.ptr(f1ao_core), k.ptrs(el) if el is not None else None, k.ptr(s1ao), natm,
            k.ptrs(outs[0]), k.ptrs(outs[1]), k.ptrs(outs[2])))
        if self.nspin == 1:
            return tuple(o[0] for o in outs)
        return tuple(outs)

    def finalize_cphf(self, f1mo, s1mo, mo1):
        """``finalize_cphf``: returns ``(mo1, mo_e1)``."""
        f1, uhf = self._spins(f1mo)
        s1, _ = self._spins(s1mo)
        m1, _ = self._spins(mo1)
        natm = int(np.prod(_shape(f1[0])[2:])) // 3
        m1 = [np.array(v, order="F", dtype=np.float64, copy=True) for v in m1]
        e1 = [np.zeros((self.nocc[s], self.nocc[s]) + tuple(_shape(f1[s])[2:]), order="F")
              for s in range(len(f1))]
        k = _Keep()
        self._check(self.lib.cphf_finalize_cphf(self.h, k.ptrs(f1), k.ptrs(s1), natm, k.ptrs(m1), k.ptrs(e1)))
        return (m1, e1) if uhf else (m1[0], e1[0])

    def get_cphf_hess(self, f1mo, s1mo, mo1, mo_e1):
        """``get_cphf_hess``: ``de [3, 3, natm, natm]``."""
        f1, _ = self._spins(f1mo)
        s1, _ = self._spins(s1mo)
        m1, _ = self._spins(mo1)
        e1, _ = self._spins(mo_e1)
        natm = int(np.prod(_shape(f1[0])[2:])) // 3
        de = np.zeros((3, 3, natm, natm), order="F")
        k = _Keep()
        self._check(self.lib.cphf_get_cphf_hess(self.h, k.ptrs(f1), k.ptrs(s1), k.ptrs(m1), k.ptrs(e1), natm,
                                                k.ptr(de)))
        return de

    # -- solver ------------------------------------------------------------------------------
    def krylov_block(self, aop, b, x0=None, tol=1e-8, max_cycle=42, max_space=14, lindep=1e-14):
        """``krylov_block`` on the GPU.  ``aop`` is a dense ``[n, n]`` matrix (applied on the
        device) or a callable mapping a host ``[n, nblock]`` array to ``A x``."""
        b = np.asfortranarray(b, dtype=np.float64)
        n, nset = b.shape
        x = np.zeros((n, nset), order="F")
        k = _Keep()
        st = Stats()
        if isinstance(aop, np.ndarray):
            op = ctypes.c_void_p()
            self._check(self.lib.cphf_dense_op_create(self.h, k.ptr(aop), n, ctypes.byref(op)))
            fn = ctypes.cast(self.lib.cphf_dense_op_apply, ctypes.c_void_p).value
            cb = AOP_FN(fn)
            user = op
        else:
            op = None
            errors = []

            def _tramp(user, xp, nn, nblock, yp, stream):
                try:
                    hx = np.zeros((nn, nblock), order="F")
                    self._check(self.lib.cphf_copy(self.h, ctypes.c_void_p(hx.ctypes.data), ctypes.c_void_p(xp),
                                                   hx.nbytes))
                    hy = np.asfortranarray(aop(hx), dtype=np.float64)
                    self._check(self.lib.cphf_copy(self.h, ctypes.c_void_p(yp), ctypes.c_void_p(hy.ctypes.data),
                                                   hy.nbytes))
                    return 0
                except Exception as e:  # reported through the status code
                    errors.append(e)
                    return 1

            cb = AOP_FN(_tramp)
            user = None
        try:
            status = self.lib.cphf_krylov_block(self.h, cb, user, k.ptr(b), k.ptr(x0), n, nset, tol, max_cycle,
                                                max_space, lindep, k.ptr(x), ctypes.byref(st))
        finally:
            if op is not None:
                self.lib.cphf_dense_op_destroy(op)
        self.last_stats = st.as_dict()
        self._check(status)
        return x

    # -- learned initial guess / preconditioner ---------------------------------------------
    def set_mlp_weights(self, weights):
        w = np.ascontiguousarray(weights, dtype=np.float32)
        self._check(self.lib.cphf_mlp_set_weights(self.h, ctypes.c_void_p(w.ctypes.data), w.size))

    def mlp_weights(self):
        w = np.zeros(MLP_NWEIGHTS, dtype=np.float32)
        self._check(self.lib.cphf_mlp_get_weights(self.h, ctypes.c_void_p(w.ctypes.data), w.size))
        return w

    def mlp_features(self, rhs):
        """Features [n, 3] (gap, b, (ia|ia)) of every vir-occ sample of ``rhs``."""
        xs, _ = self._spins(rhs)
        nprop = _nprop(_shape(xs[0]))
        k = _Keep()
        n = ctypes.c_int64()
        p = k.ptrs(xs)
        self._check(self.lib.cphf_mlp_features(self.h, p, nprop, None, 0, ctypes.byref(n)))
        feat = np.zeros((n.value, 3), dtype=np.float32)
        self._check(self.lib.cphf_mlp_features(self.h, p, nprop, ctypes.c_void_p(feat.ctypes.data), n.value,
                                               ctypes.byref(n)))
        return feat

    def mlp_forward(self, feat, bf16=False):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        out = np.zeros((feat.shape[0], 2), dtype=np.float32)
        self._check(self.lib.cphf_mlp_forward(self.h, ctypes.c_void_p(feat.ctypes.data), feat.shape[0],
                                              ctypes.c_void_p(out.ctypes.data), 1 if bf16 else 0))
        return out

    def mlp_loss_grad(self, feat, target):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        grad = np.zeros(MLP_NWEIGHTS, dtype=np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.cphf_mlp_loss_grad(self.h, ctypes.c_void_p(feat.ctypes.data),
                                                ctypes.c_void_p(target.ctypes.data), feat.shape[0],
                                                ctypes.byref(loss), ctypes.c_void_p(grad.ctypes.data)))
        return loss.value, grad

    def mlp_train(self, feat, target, epochs=20, batch=4096, lr=1e-3, seed=0):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        hist = np.zeros(max(epochs, 1), dtype=np.float32)
        self._check(self.lib.cphf_mlp_train(self.h, ctypes.c_void_p(feat.ctypes.data),
                                            ctypes.c_void_p(target.ctypes.data), feat.shape[0], epochs, batch,
                                            lr, seed, ctypes.c_void_p(hist.ctypes.data)))
        return hist[:epochs]
