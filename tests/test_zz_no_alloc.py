"""The allocation-free RI-J entry point, for callers that cannot allocate device memory.

Runs last (file name) so that a failure here cannot hide any other test's result.  It calls
``cphf_rij_response_bra_noalloc`` through the C ABI with device buffers owned by the test
and compares it, on two calls in a row, with the regular RI-JK plugin entry point
(``cphf_plugin_response_bra`` with scale_k = 0, i.e. the Coulomb part alone).
"""

import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_noalloc_rij_matches_plugin_entry_point():
    import torch
    from cphf_gb300 import Context, load_library, synth
    from oracle.rijk import unpack_tri_sym

    lib = load_library()
    lib.cphf_rij_response_bra_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p,
                                                   ctypes.c_void_p]
    lib.cphf_rij_response_bra_noalloc.restype = ctypes.c_int32
    lib.cphf_rij_noalloc_capacity.restype = ctypes.c_int64
    cap = lib.cphf_rij_noalloc_capacity()

    s = synth.make_system(dict(nao=72, naux=230, nocc=(9,), natm=5, decay=10.0), seed=31, scale_k=0.0)
    nao, naux, no = s.nao, s.naux, s.nocc[0]
    ctx = Context()
    ctx.set_cderi(s.cderi, s.scale_j, 0.0)
    ctx.make_response_preparation(s.mo_coeff[0], s.mo_occ[0], s.mo_energy[0])

    # Z[mu, i, P] = sum_nu B_P[mu, nu] Cocc[nu, i], the input the caller provides
    cd = unpack_tri_sym(s.cderi, nao)
    Z = np.einsum("uvP,vi->uiP", cd, s.mo_coeff[0][:, :no], optimize=True)
    dev = torch.device("cuda:0")
    Zd = torch.from_numpy(np.ascontiguousarray(Z.transpose(2, 1, 0))).to(dev)   # col-major [nao, nocc, naux]
    rng = np.random.default_rng(32)
    for call in range(2):
        nb = 11 + 6 * call
        assert naux * nb <= cap
        bra = rng.standard_normal((nao, no, nb))
        ref = ctx.get_response_bra(bra, plugin="rijk")
        bra_d = torch.from_numpy(np.ascontiguousarray(bra.transpose(2, 1, 0))).to(dev)
        out_d = torch.full((nb, no, nao), np.nan, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream().cuda_stream
        st = lib.cphf_rij_response_bra_noalloc(ctypes.c_void_p(Zd.data_ptr()), ctypes.c_void_p(bra_d.data_ptr()),
                                               nao, no, naux, nb, s.scale_j, ctypes.c_void_p(out_d.data_ptr()),
                                               ctypes.c_void_p(stream))
        assert st == 0
        torch.cuda.synchronize()
        got = out_d.cpu().numpy().transpose(2, 1, 0)
        assert rel_err(got, ref) < 1e-12

    # sizes beyond the static scratch are rejected, not truncated
    nb_big = cap // naux + 1
    st = lib.cphf_rij_response_bra_noalloc(ctypes.c_void_p(Zd.data_ptr()), ctypes.c_void_p(Zd.data_ptr()), nao, no,
                                           naux, nb_big, 1.0, ctypes.c_void_p(Zd.data_ptr()), None)
    assert st == 8
