"""C-ABI library: it loads without a GPU and exports every entry point that
include/nfft_gb300.h declares, with the binding's signatures.  No compute
calls are made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nfft_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nfft_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import nfftgb300
    if not os.path.exists(nfftgb300.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return nfftgb300.load()


def test_library_exports_header(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    import nfftgb300
    assert set(declared_functions()) == set(nfftgb300.exported_symbols())


def test_status_strings_and_defaults(lib):
    import nfftgb300._lib as L
    assert lib.nfft_status_string(0) == b"ok"
    assert lib.nfft_status_string(L.NFFT_ERR_DIM_MISMATCH) == b"dimension mismatch"
    prm = L.nfft_params()
    lib.nfft_params_default(ctypes.byref(prm))
    assert (prm.m, prm.sigma, prm.window, prm.precompute, prm.blocking) == (4, 2.0, 0, 4, 1)


def test_plan_create_rejects_bad_arguments_without_gpu(lib):
    """Argument validation happens before any device call."""
    import nfftgb300._lib as L
    prm = L.nfft_params()
    lib.nfft_params_default(ctypes.byref(prm))
    h = ctypes.c_void_p()
    N = (ctypes.c_int64 * 3)(16, 16, 1)
    assert lib.nfft_plan_create(ctypes.byref(h), 16, 2, N, 10, ctypes.byref(prm), None) == L.NFFT_ERR_INVALID_ARG
    assert lib.nfft_plan_create(ctypes.byref(h), 32, 4, N, 10, ctypes.byref(prm), None) == L.NFFT_ERR_UNSUPPORTED
    prm.m = 9
    assert lib.nfft_plan_create(ctypes.byref(h), 32, 2, N, 10, ctypes.byref(prm), None) == L.NFFT_ERR_UNSUPPORTED
    assert b"m = 9" in lib.nfft_last_error()
    prm.m = 4
    prm.window = 7
    assert lib.nfft_plan_create(ctypes.byref(h), 32, 2, N, 10, ctypes.byref(prm), None) == L.NFFT_ERR_UNSUPPORTED
    prm.window = 0
    prm.precompute = 0
    assert lib.nfft_plan_create(ctypes.byref(h), 32, 2, N, 10, ctypes.byref(prm), None) == L.NFFT_ERR_UNSUPPORTED
    assert not h.value


def test_julia_backend_binds_the_interface_entry_points():
    """The Julia ccall backend (not executable here: no Julia) binds every
    entry point the AbstractNFFTs interface, directional plans and batches
    need; the remaining header functions are inspection / tuning helpers."""
    jl = open(os.path.join(ROOT, "nfft.jl_gb300", "julia", "src", "NFFTGB300.jl")).read()
    helpers = {"nfft_bin_nodes_noalloc", "nfft_get_binning", "nfft_get_deconv_factors", "nfft_get_timing_totals",
               "nfft_kernel_launch_count", "nfft_params_default", "nfft_plan_copy", "nfft_set_block_size",
               "nfft_sync", "nfft_timing_reset"}
    for n in declared_functions():
        if n not in helpers:
            assert f":{n}" in jl, n


def test_julia_chainrules_extension():
    """The Julia backend's ChainRulesCore extension (not executable here: no
    Julia) is declared in Project.toml and defines the rrules of nfft and
    nfft_adjoint (AbstractNFFTs/ext/AbstractNFFTsChainRulesCoreExt.jl:31-61)
    with a node tangent from the library's node-gradient kernel instead of
    NoTangent."""
    jdir = os.path.join(ROOT, "nfft.jl_gb300", "julia")
    proj = open(os.path.join(jdir, "Project.toml")).read()
    assert "ChainRulesCore" in proj and 'NFFTGB300ChainRulesCoreExt = "ChainRulesCore"' in proj
    ext = open(os.path.join(jdir, "ext", "NFFTGB300ChainRulesCoreExt.jl")).read()
    assert "ChainRulesCore.rrule(::typeof(AbstractNFFTs.nfft), k::AbstractMatrix" in ext
    assert "ChainRulesCore.rrule(::typeof(AbstractNFFTs.nfft_adjoint), k::AbstractMatrix" in ext
    assert ext.count("NFFTGB300.grad_nodes!(dk, p,") == 2
    # the node tangent is projected, not NoTangent, in both pullbacks
    assert ext.count("project_k(Array(dk))") == 2
    src = open(os.path.join(jdir, "src", "NFFTGB300.jl")).read()
    assert "function grad_nodes!(" in src and ":nfft_grad_nodes" in src


def test_build_compiles_every_source():
    """build() compiles every CUDA source of the package (a file missing from
    the list would silently drop its entry points on the GPU machine)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "nfft.jl_gb300"))
    import build as B
    on_disk = sorted(f for f in os.listdir(B.CSRC) if f.endswith(".cu"))
    assert sorted(B.SOURCES) == on_disk
