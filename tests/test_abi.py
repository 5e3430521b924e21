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


BINDING = os.path.join(ROOT, "jurassic_gb300", "binding", "jurassic_unified_library.c")
REFABI = os.path.join(ROOT, "tests", "refabi")
DIMS = ["-DND=16", "-DNG=4", "-DNW=2", "-DNP=128", "-DNR=16", "-DNCL=8", "-DNSF=8", "-DLEN=4096"]


def _reference_src():
    from oracle import refimpl
    d = os.path.join(refimpl.source_dir() or "", "src")
    return d if os.path.isfile(os.path.join(d, "jurassic.h")) else None


def _cc():
    import shutil
    return shutil.which("gcc") or shutil.which("cc")


def test_binding_compiles_against_reference_header(tmp_path):
    """The reference-side binding (jur_unified_init,
    jur_unified_formod_multiple_packages, the kernel() and
    optimal_estimation drop-ins; the seam of formod.c:26-27, 60-76) compiles
    against the reference's own jurassic.h (its ctl_t, atm_t, obs_t,
    dimensions and GSL types) and this library's header, warnings as errors,
    with the reference's default dimensions and with small ones.  Skipped
    where the reference tree is absent."""
    import subprocess
    src_dir, cc = _reference_src(), _cc()
    if cc is None or src_dir is None:
        pytest.skip("reference tree or C compiler not available")
    for dims in ([], DIMS):
        r = subprocess.run([cc, "-std=gnu99", "-Wall", "-Wextra", "-Werror", "-fopenmp"] + dims +
                           ["-isystem", src_dir, "-isystem", os.path.join(ROOT, "oracle", "gsl_shim"),
                            "-I", os.path.join(ROOT, "include"), "-c", BINDING,
                            "-o", str(tmp_path / "binding.o")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


RET_PATCH = r"""
/* the reference's retrieval driver with the optimal_estimation drop-in: its
   own ret_t filled into a jgb_ret by the binding's macro */
#define main jref_retrieval_main_unused
#include "retrieval.c"
#undef main
#include "jurassic_unified_library.h"
void retrieve_on_gpu(ret_t *ret, obs_t *obs_meas, obs_t *obs_i, atm_t *atm_apr, atm_t *atm_i,
                     gsl_matrix *cov) {
  jgb_ret r;
  JUR_UNIFIED_RET_FROM(ret, &r);
  jur_unified_optimal_estimation(&r, obs_meas, obs_i, atm_apr, atm_i, cov);
}
"""


def test_ret_conversion_compiles_inside_reference_retrieval(tmp_path):
    """JUR_UNIFIED_RET_FROM expands against the reference's own ret_t (it is
    private to retrieval.c, so the test compiles retrieval.c with a function
    that uses the macro appended), warnings in the added code as errors."""
    import subprocess
    src_dir, cc = _reference_src(), _cc()
    if cc is None or src_dir is None:
        pytest.skip("reference tree or C compiler not available")
    src = tmp_path / "ret_patch.c"
    src.write_text(RET_PATCH)
    r = subprocess.run([cc, "-std=gnu99", "-fopenmp", "-Werror=incompatible-pointer-types",
                        "-Werror=int-conversion", "-Werror=implicit-function-declaration",
                        "-isystem", src_dir, "-I", src_dir,
                        "-isystem", os.path.join(ROOT, "oracle", "gsl_shim"),
                        "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "jurassic_gb300", "binding"), "-c", str(src),
                        "-o", str(tmp_path / "ret_patch.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


LAYOUT_PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "jurassic.h"
#define F(T, m) printf("%s.%s %zu %zu\n", #T, #m, offsetof(T, m), sizeof(((T *)0)->m))
int main(void) {
  printf("atm_t %zu\nobs_t %zu\nctl_t %zu\n", sizeof(atm_t), sizeof(obs_t), sizeof(ctl_t));
  F(atm_t, np); F(atm_t, time); F(atm_t, z); F(atm_t, lon); F(atm_t, lat); F(atm_t, p);
  F(atm_t, t); F(atm_t, q); F(atm_t, k); F(atm_t, clz); F(atm_t, cldz); F(atm_t, clk);
  F(atm_t, sfz); F(atm_t, sfp); F(atm_t, sft); F(atm_t, sfeps);
  F(obs_t, nr); F(obs_t, time); F(obs_t, obsz); F(obs_t, obslon); F(obs_t, obslat);
  F(obs_t, vpz); F(obs_t, vplon); F(obs_t, vplat); F(obs_t, tpz); F(obs_t, tplon);
  F(obs_t, tplat); F(obs_t, tau); F(obs_t, rad);
  F(ctl_t, ng); F(ctl_t, emitter); F(ctl_t, nd); F(ctl_t, nu); F(ctl_t, nw); F(ctl_t, window);
  F(ctl_t, ncl); F(ctl_t, clnu); F(ctl_t, nsf); F(ctl_t, sfnu); F(ctl_t, sftype);
  F(ctl_t, sfsza); F(ctl_t, tblbase); F(ctl_t, tblfmt); F(ctl_t, hydz); F(ctl_t, ctm_co2);
  F(ctl_t, ctm_h2o); F(ctl_t, ctm_n2); F(ctl_t, ctm_o2); F(ctl_t, refrac); F(ctl_t, rayds);
  F(ctl_t, raydz); F(ctl_t, fov); F(ctl_t, retp_zmin); F(ctl_t, retp_zmax);
  F(ctl_t, rett_zmin); F(ctl_t, rett_zmax); F(ctl_t, retq_zmin); F(ctl_t, retq_zmax);
  F(ctl_t, retk_zmin); F(ctl_t, retk_zmax); F(ctl_t, ret_clz); F(ctl_t, ret_cldz);
  F(ctl_t, ret_clk); F(ctl_t, ret_sfz); F(ctl_t, ret_sfp); F(ctl_t, ret_sft);
  F(ctl_t, ret_sfeps); F(ctl_t, write_bbt); F(ctl_t, write_matrix); F(ctl_t, formod);
  return 0;
}
"""


def test_restated_struct_layouts_match_reference(tmp_path):
    """tests/refabi/jurassic.h (used to run the binding where the reference
    tree is absent) gives ctl_t, atm_t and obs_t the same size and member
    offsets as the reference's jurassic.h, for the dimensions the GPU test
    uses and for the reference's defaults.  Skipped where the reference tree
    is absent."""
    import subprocess
    src_dir, cc = _reference_src(), _cc()
    if cc is None or src_dir is None:
        pytest.skip("reference tree or C compiler not available")
    probe = tmp_path / "probe.c"
    probe.write_text(LAYOUT_PROBE)
    for dims in ([], DIMS):
        outs = []
        for inc in (src_dir, REFABI):
            exe = tmp_path / "probe"
            r = subprocess.run([cc, "-std=gnu99", "-w", "-fopenmp"] + dims +
                               ["-I", inc, "-isystem", os.path.join(ROOT, "oracle", "gsl_shim"),
                                str(probe), "-o", str(exe), "-lm"], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
            outs.append(subprocess.run([str(exe)], capture_output=True, text=True).stdout)
        assert outs[0] == outs[1] and len(outs[0].splitlines()) > 60, (dims, outs)


def test_binding_and_driver_build_with_restated_header(tmp_path, built_lib):
    """The binding and the GPU test's driver compile against the restated
    header and link with the library (the GPU test builds them the same way
    on the GPU machine)."""
    import subprocess
    cc = _cc()
    if cc is None:
        pytest.skip("no C compiler")
    fill = tmp_path / "fill.c"
    fill.write_text('#include "jurassic.h"\nvoid drv_fill_ctl(ctl_t *c) { c->ng = 0; }\n')
    libdir = os.path.join(ROOT, "jurassic_gb300")
    r = subprocess.run([cc, "-std=gnu99", "-fPIC", "-shared", "-Wall", "-Wextra", "-Werror"] + DIMS +
                       ["-I", REFABI, "-isystem", os.path.join(ROOT, "oracle", "gsl_shim"),
                        "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "jurassic_gb300", "binding"),
                        os.path.join(REFABI, "driver.c"), BINDING, str(fill),
                        "-o", str(tmp_path / "lib.so"), "-L", libdir, "-ljurassic_gb300",
                        "-Wl,--no-undefined", "-lm", "-Wl,-rpath," + libdir,
                        "-L/usr/local/cuda/lib64", "-lcudart"], capture_output=True, text=True)
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
