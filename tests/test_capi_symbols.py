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


def test_header_is_plain_c_and_links(built, tmp_path):
    """include/dfg.h is the C ABI a cgo / JNI / ctypes / C caller binds: it
    compiles as strict C99 without warnings, every declared entry point
    resolves when a C program links libdfg.so, and the calls that need no
    device (version, error text, the GiD reader's error path, context
    creation without a GPU) behave from C as documented, and the server
    structs' documented positional initializers still fill every field."""
    import os
    import shutil
    import torch
    from delfem_gb300 import capi
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    names = capi.header_symbols()
    src = tmp_path / "abi.c"
    refs = "\n".join(f"  (entry_fn)&{n}," for n in names)
    gpu = 1 if torch.cuda.is_available() else 0
    src.write_text(f"""#include <stdio.h>
#include <string.h>
#include "dfg.h"

typedef void (*entry_fn)(void);
static const entry_fn entry_points[] = {{
{refs}
}};

int main(void) {{
  /* the positional initializers documented for the server */
  dfg_server_config cfg = {{DFG_PREC_FP32_FACTOR, 1e-8, 20000, 0, 128, 8, 0, 0, 0, 0}};
  dfg_request q = {{4, 0, 0, NULL, NULL, NULL, NULL, 5, NULL, NULL, NULL}};
  size_t i;
  int nd = 0, nn = 0, nv = 0, ne = 0;
  dfg_ctx ctx = NULL;
  for (i = 0; i < sizeof entry_points / sizeof entry_points[0]; ++i)
    if (!entry_points[i]) return 10;
  if (cfg.size_groups != 0 || q.nparams != 5 || q.x_out != NULL) return 16;
  if (strncmp(dfg_version(), "dfg", 3) != 0) return 11;
  if (dfg_last_error(NULL) == NULL) return 12;
  if (dfg_mesh_read_gid("{tmp_path}/missing.msh", &nd, &nn, &nv, &ne, NULL, NULL) != DFG_INVALID_ARGUMENT) return 13;
  if (strstr(dfg_last_error(NULL), "dfg_mesh_read_gid") == NULL) return 14;
  if (!{gpu} && dfg_ctx_create(0, &ctx) == DFG_OK) return 15;
  printf("%u entry points\\n", (unsigned)(sizeof entry_points / sizeof entry_points[0]));
  return 0;
}}
""")
    exe = tmp_path / "abi"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{root}/include", str(src),
                    built, f"-Wl,-rpath,{os.path.dirname(built)}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.strip() == f"{len(names)} entry points"
