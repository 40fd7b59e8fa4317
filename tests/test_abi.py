"""CPU tests of the C ABI boundary: the in-tree library loads and exports every declared symbol."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mpsg.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mpsg_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("mpsg_contract_twosite", "mpsg_add_contraction_layer", "mpsg_split2", "mpsg_lanczos2",
                 "mpsg_dmrg_simulate", "mpsg_tensor_create"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from mpstools_gb300 import build as B
    lib = B.build()
    L = ctypes.CDLL(lib)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_context_creation_fails_cleanly_without_gpu():
    """No GPU here: context creation must return an error code, not abort."""
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("GPU present")
    from mpstools_gb300 import lib
    L = lib.load()
    h = ctypes.c_void_p()
    rc = L.mpsg_ctx_create(0, ctypes.byref(h))
    assert rc != 0
    assert len(L.mpsg_last_error()) > 0


def test_itokey_and_mpo_marshalling():
    from mpstools_gb300 import lib, models as M
    w = M.heisenberg_mpo(np.ones(3), np.ones(3), np.zeros(4))[1]
    arg = lib.MPOArg(w)
    assert arg.s.nterms == len(w[0]) and arg.s.Dl == 5 and arg.s.Dr == 5
    k = lib.ItoKeyArg([0, 1])
    assert k.s.d == 2


def test_header_is_plain_c(tmp_path):
    """include/mpsg.h compiles as C99 and as C++ (an FFI or a C host can include it as it is)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use_header.c"
    src.write_text('#include "mpsg.h"\nint main(void) { return (int)sizeof(mpsg_prec) == 0; }\n')
    for lang, std in (("c", "-std=c99"), ("c++", "-std=c++17")):
        r = subprocess.run([cc, "-x", lang, std, "-Wall", "-Werror", "-pedantic", "-fsyntax-only",
                            "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
        assert r.returncode == 0, (lang, r.stderr)


def test_plain_c_host_links_and_calls_the_library(tmp_path):
    """A C program links libmpsg.so and calls it: without a GPU context creation returns a status and
    a message instead of aborting; with one it creates and destroys a context."""
    import shutil
    import subprocess
    from mpstools_gb300 import build as B
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = B.build()
    src = tmp_path / "host.c"
    src.write_text(r'''
#include <stdio.h>
#include "mpsg.h"
int main(void) {
  mpsg_ctx ctx = 0;
  mpsg_status rc = mpsg_ctx_create(0, &ctx);
  if (rc == MPSG_OK) { mpsg_ctx_destroy(ctx); printf("context ok\n"); return 0; }
  printf("status %d: %s\n", (int)rc, mpsg_last_error());
  return mpsg_last_error()[0] ? 0 : 1;
}
''')
    exe = tmp_path / "host"
    libdir = os.path.dirname(lib)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe), "-L", libdir, "-lmpsg", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert r.stdout.startswith(("context ok", "status "))
