"""The C ABI without a GPU: the library loads, exports every declared symbol, and the host-only
entry points behave (defaults of HessSCFConfig, status strings, clean failure without a device)."""

import ctypes
import re

import pytest

from conftest import REPO, gpu_available


def declared_symbols():
    text = (REPO / "include" / "cphf.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cphf_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for name in ["cphf_rijk_set_cderi", "cphf_xc_set_grid", "cphf_prepare", "cphf_response_bra",
                 "cphf_solve_dimless_cphf", "cphf_krylov_block", "cphf_finalize_cphf", "cphf_get_cphf_hess"]:
        assert name in syms


def test_library_exports_every_declared_symbol(built_lib):
    missing = [s for s in declared_symbols() if not hasattr(built_lib, s)]
    assert not missing, missing


def test_python_binding_covers_exports(built_lib):
    from cphf_gb300 import EXPORTS
    assert set(EXPORTS) <= set(declared_symbols())
    assert set(declared_symbols()) <= set(EXPORTS)


def test_config_defaults_mirror_hess_scf_config(built_lib):
    from cphf_gb300 import Config
    cfg = Config()
    assert built_lib.cphf_config_default(ctypes.byref(cfg)) == 0
    # HessSCFConfig::default (src/hessian/rscf.rs:14-18)
    assert cfg.level_shift == 0.0
    assert cfg.cphf_tol == 1e-8
    assert cfg.cphf_max_cycle == 42
    assert cfg.cphf_max_space == 14
    assert cfg.cphf_lindep == 1e-14
    assert cfg.precision == 0
    assert built_lib.cphf_config_default(None) != 0


def test_status_strings(built_lib):
    assert built_lib.cphf_status_string(2) == b"krylov_block failed to converge"
    assert built_lib.cphf_status_string(0) == b"ok"


@pytest.mark.skipif(gpu_available(), reason="checks the no-device failure path")
def test_context_creation_fails_loudly_without_gpu(built_lib):
    from cphf_gb300 import Context, CphfError
    with pytest.raises(CphfError):
        Context()


def test_null_context_is_rejected(built_lib):
    assert built_lib.cphf_ctx_synchronize(None) == 8
    assert built_lib.cphf_ctx_destroy(None) == 0
