"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares (no compute calls here)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(jgb_[A-Za-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("jgb_create", "jgb_destroy", "jgb_formod", "jgb_formod_batch",
                     "jgb_formod_batch_dev", "jgb_set_table", "jgb_set_filter"):
        assert required in names


def test_library_exports_all_declared_symbols(built_lib):
    lib = ctypes.CDLL(os.path.join(ROOT, "jurassic_gb300", "libjurassic_gb300.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, "not exported: %s" % missing


def test_python_binding_covers_header(built_lib):
    from jurassic_gb300 import native
    missing = [n for n in declared_functions() if n not in native.SIGNATURES]
    assert not missing, "no ctypes signature for: %s" % missing


def test_invalid_control_is_rejected_without_gpu(built_lib):
    """Argument checks run before any device work: a bad control set returns
    JGB_ERR_ARG (the reference would exit())."""
    from jurassic_gb300 import native
    L = native.load()
    c = native._Ctl(ng=-1, nd=0)
    h = ctypes.c_void_p()
    assert L.jgb_create(ctypes.byref(c), 0, ctypes.byref(h)) == 1
    assert not h.value


C_CONSUMER = r"""
/* A C99 consumer of the ABI: the header compiles as C, the library links,
   and host-only calls run (no device work). */
#include <stdio.h>
#include <string.h>
#include "jurassic_gb300.h"

static int same(int np, const double *p, const int *nt, const double *t, const int *nu,
                const float *u, const float *e, const double *p2, const int *nt2,
                const double *t2, const int *nu2, const float *u2, const float *e2) {
  int ip, it;
  for (ip = 0; ip < np; ip++) {
    if (p[ip] != p2[ip] || nt[ip] != nt2[ip]) return 0;
    for (it = 0; it < nt[ip]; it++) {
      int r = ip * 2 + it;
      if (t[r] != t2[r] || nu[r] != nu2[r]) return 0;
      if (memcmp(u + r * 3, u2 + r * 3, sizeof(float) * nu[r]) != 0) return 0;
      if (memcmp(e + r * 3, e2 + r * 3, sizeof(float) * nu[r]) != 0) return 0;
    }
  }
  return 1;
}

int main(int argc, char **argv) {
  double p[2] = {1.0, 10.0}, t[4] = {200.0, 250.0, 220.0, 0.0};
  int nt[2] = {2, 1}, nu[4] = {3, 2, 3, 0};
  float u[12], e[12];
  double p2[2], t2[4];
  int nt2[2], nu2[4], np2 = -1, fmt, i;
  float u2[12], e2[12];
  jgb_ctl c;
  jgb_ctx *ctx = NULL;
  char path[4096];
  if (argc < 2) return 1;
  for (i = 0; i < 12; i++) {
    u[i] = 1e18f * (float)(i % 3 + 1);
    e[i] = 0.1f * (float)(i % 3 + 1);
  }
  for (fmt = 1; fmt <= 2; fmt++) {
    snprintf(path, sizeof path, "%s.%d", argv[1], fmt);
    if (jgb_write_table_file(path, fmt, 2, p, nt, t, nu, u, e, 2, 3) != JGB_OK) return 2;
    if (jgb_read_table_file(path, fmt, 2, 2, 3, &np2, p2, nt2, t2, nu2, u2, e2) != JGB_OK) return 3;
    if (np2 != 2 || !same(2, p, nt, t, nu, u, e, p2, nt2, t2, nu2, u2, e2)) return 4;
  }
  memset(&c, 0, sizeof c);
  c.ng = -1;
  if (jgb_create(&c, 0, &ctx) != JGB_ERR_ARG || ctx != NULL) return 5;
  if (jgb_read_table_file(path, 3, 2, 2, 3, &np2, p2, nt2, t2, nu2, u2, e2) != JGB_ERR_ARG) return 6;
  puts("ok");
  return 0;
}
"""


def test_c_consumer_compiles_links_and_runs(tmp_path, built_lib):
    """The header compiles as strict C99 (the reference is C), a C program
    links against the library, and its host-only calls (table files, the
    argument checks of jgb_create) run without a GPU."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from jurassic_gb300 import native
    src = tmp_path / "consumer.c"
    src.write_text(C_CONSUMER)
    exe = tmp_path / "consumer"
    libdir = os.path.dirname(native.LIB_PATH)
    r = subprocess.run([cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-ljurassic_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ)
    cuda_lib = "/usr/local/cuda/lib64"
    env["LD_LIBRARY_PATH"] = ":".join(x for x in (env.get("LD_LIBRARY_PATH", ""), cuda_lib) if x)
    r = subprocess.run([str(exe), str(tmp_path / "tbl")], capture_output=True, text=True, env=env)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)


def test_integration_binding_compiles_against_reference_header(tmp_path):
    """The binding shown in INTEGRATION.md (jur_unified_init and
    jur_unified_formod_multiple_packages on top of this library, the seam of
    formod.c:60-76) compiles against the reference's own jurassic.h (its
    ctl_t, atm_t, obs_t and dimensions) and this header, warnings as errors.
    Skipped where the reference tree is absent."""
    import shutil
    import subprocess
    from oracle import refimpl
    cc = shutil.which("gcc") or shutil.which("cc")
    src_dir = os.path.join(refimpl.source_dir() or "", "src")
    if cc is None or not os.path.isfile(os.path.join(src_dir, "jurassic.h")):
        pytest.skip("reference tree or C compiler not available")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    start = text.index("/* jurassic_unified_library.c")
    code = text[start:text.index("```", start)]
    src = tmp_path / "jurassic_unified_library.c"
    src.write_text(code)
    r = subprocess.run([cc, "-std=gnu99", "-Wall", "-Wextra", "-Werror", "-fopenmp",
                        "-isystem", src_dir, "-isystem", os.path.join(ROOT, "oracle", "gsl_shim"),
                        "-I", os.path.join(ROOT, "include"), "-c", str(src),
                        "-o", str(tmp_path / "binding.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_new_entry_points_check_arguments_without_gpu(built_lib):
    """Bad arguments of the table-file, measurement and self-test entry
    points return JGB_ERR_ARG before any device work."""
    from jurassic_gb300 import native
    L = native.load()
    n = ctypes.c_int(0)
    assert L.jgb_read_table_file(None, 2, 1, 1, 1, ctypes.byref(n), None, None, None, None,
                                 None, None) == native.ERR_ARG
    p = (ctypes.c_double * 1)(1.0)
    nt = (ctypes.c_int * 1)(3)          # more temperatures than the capacity
    t = (ctypes.c_double * 2)(200.0, 210.0)
    nu = (ctypes.c_int * 2)(1, 1)
    u = (ctypes.c_float * 2)(1.0, 2.0)
    e = (ctypes.c_float * 2)(0.1, 0.2)
    assert L.jgb_write_table_file(b"/nonexistent/x.bin", 2, 1, p, nt, t, nu, u, e, 2, 1) == \
        native.ERR_ARG
    assert L.jgb_write_table_file(b"/nonexistent/x.bin", 5, 0, None, None, None, None, None,
                                  None, 2, 1) == native.ERR_ARG
    g = ctypes.c_double(0.0)
    assert L.jgb_measure_l2_read(0, 1, ctypes.byref(g)) == native.ERR_ARG
    assert L.jgb_measure_l2_read(1 << 20, 0, ctypes.byref(g)) == native.ERR_ARG
    assert L.jgb_selftest_bounded_wait(0, 0, None, None) == native.ERR_ARG
    assert L.jgb_read_tables(None, b"tbl", 2) == native.ERR_ARG
