"""The C-ABI library loads without a GPU and exports every entry point
include/dfg.h declares; the Python binding covers exactly that set."""
import subprocess

import pytest


@pytest.fixture(scope="module")
def built():
    from delfem_gb300 import build as B
    return B.build()


def test_library_exports_every_declared_symbol(built):
    from delfem_gb300 import capi
    L = capi.lib()
    declared = capi.header_symbols()
    assert len(declared) >= 40
    for name in declared:
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert set(declared) <= exported


def test_binding_matches_header():
    from delfem_gb300 import capi
    assert set(capi.SIGNATURES) == set(capi.header_symbols())


def test_version_and_error_text_without_gpu(built):
    from delfem_gb300 import capi
    L = capi.lib()
    assert L.dfg_version().startswith(b"dfg")
    assert isinstance(L.dfg_last_error(None), bytes)


def test_context_creation_fails_cleanly_without_device(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from delfem_gb300 import capi, linsys
    with pytest.raises(capi.DfgError):
        linsys.Context(0)


def test_library_has_no_undefined_symbols_of_its_own(built):
    """A source left out of the build links anyway (shared objects may carry
    undefined symbols) and fails only at load time; catch it here."""
    out = subprocess.run(["nm", "-D", "--undefined-only", "-C", built], capture_output=True, text=True,
                         check=True).stdout
    ours = [ln for ln in out.splitlines() if "dfg" in ln]
    assert not ours, ours
