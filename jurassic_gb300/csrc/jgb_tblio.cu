// Emissivity table files of the reference, read and written on the host:
// read_tbl (src/jurassic.c:4949-5110) and write_tbl (src/jurassic.c:
// 5810-5892), ASCII (TBLFMT 1) and binary (TBLFMT 2), plus the loader that
// reads every (channel, emitter) file of a context and uploads it into the
// device layout (jgb_set_table).  Reading one format and writing the other
// converts between them (the reference's tblfmt tool).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/jurassic_gb300.h"
#include "jgb_ctx.h"
#include "jgb_internal.h"

namespace {

// accepted ranges of an ASCII table point (UMIN, UMAX, EPSMIN, EPSMAX,
// jurassic.h:264-339)
constexpr double kUmin = 0.0, kUmax = 1e30, kEpsmin = 0.0, kEpsmax = 1.0;

// One table in caller arrays with the row layout of tbl_t:
// p[tp], nt[tp], t[tp][tt], nu[tp][tt], u/eps[tp][tt][tu].
struct TblView {
  int tp, tt, tu;
  double* p;
  int* nt;
  double* t;
  int* nu;
  float* u;
  float* eps;
};

void clear(const TblView& v) {
  std::memset(v.p, 0, sizeof(double) * v.tp);
  std::memset(v.nt, 0, sizeof(int) * v.tp);
  std::memset(v.t, 0, sizeof(double) * (size_t)v.tp * v.tt);
  std::memset(v.nu, 0, sizeof(int) * (size_t)v.tp * v.tt);
  std::memset(v.u, 0, sizeof(float) * (size_t)v.tp * v.tt * v.tu);
  std::memset(v.eps, 0, sizeof(float) * (size_t)v.tp * v.tt * v.tu);
}

// ASCII table (TBLFMT 1, jurassic.c:4991-5047): lines "p T u eps"; a line
// that does not start with four numbers is skipped, as is a point outside
// the accepted ranges; a new pressure opens a new pressure level, a new
// temperature a new temperature row (so does the first point of a pressure
// level, whose temperature index the reference would otherwise leave at
// -1); within a row a point is appended only if both u and eps exceed the
// last appended point (of any row), otherwise it overwrites that point.
int read_ascii(FILE* f, const TblView& v, int* np_out, std::string& msg) {
  std::vector<char> line(1 << 16);
  int ip = -1, it = -1, iu = -1;
  double p_old = -999, t_old = -999, u_old = -999, e_old = -999;
  while (std::fgets(line.data(), (int)line.size(), f)) {
    const size_t len = std::strlen(line.data());
    if (len + 1 == line.size() && line[len - 1] != '\n') {  // drop the rest of a long line
      int ch;
      while ((ch = std::fgetc(f)) != EOF && ch != '\n') {
      }
    }
    double press, temp, u, eps;
    if (std::sscanf(line.data(), "%lg %lg %lg %lg", &press, &temp, &u, &eps) != 4) continue;
    if (u < kUmin || u > kUmax || eps < kEpsmin || eps > kEpsmax) continue;
    if (press != p_old) {
      p_old = press;
      if (++ip >= v.tp) {
        msg = "Too many pressure levels!";
        return JGB_ERR_ARG;
      }
      it = -1;
    }
    if (temp != t_old || it < 0) {
      t_old = temp;
      if (++it >= v.tt) {
        msg = "Too many temperatures!";
        return JGB_ERR_ARG;
      }
      iu = -1;
    }
    if ((eps > e_old && u > u_old) || iu < 0) {
      e_old = eps;
      u_old = u;
      if (++iu >= v.tu) {
        msg = "Too many column densities!";
        return JGB_ERR_ARG;
      }
    }
    const size_t r = (size_t)ip * v.tt + it;
    v.p[ip] = press;
    v.t[r] = temp;
    v.u[r * v.tu + iu] = (float)u;
    v.eps[r * v.tu + iu] = (float)eps;
    v.nt[ip] = it + 1;
    v.nu[r] = iu + 1;
  }
  *np_out = ip + 1;
  return JGB_OK;
}

template <typename T>
bool take(FILE* f, T* dst, size_t n) {
  return std::fread(dst, sizeof(T), n, f) == n;
}

// Binary table (TBLFMT 2, jurassic.c:5050-5082): int np, double p[np]; per
// pressure int nt, double t[nt]; per temperature int nu, float u[nu],
// float eps[nu] (native little-endian, as the reference writes it).
int read_binary(FILE* f, const TblView& v, int* np_out, std::string& msg) {
  int np = 0;
  if (!take(f, &np, 1) || np < 0) {
    msg = "truncated table file";
    return JGB_ERR_IO;
  }
  if (np > v.tp) {
    msg = "Too many pressure levels!";
    return JGB_ERR_ARG;
  }
  if (!take(f, v.p, (size_t)np)) {
    msg = "truncated table file";
    return JGB_ERR_IO;
  }
  for (int ip = 0; ip < np; ip++) {
    int nt = 0;
    if (!take(f, &nt, 1) || nt < 0) {
      msg = "truncated table file";
      return JGB_ERR_IO;
    }
    if (nt > v.tt) {
      msg = "Too many temperatures!";
      return JGB_ERR_ARG;
    }
    v.nt[ip] = nt;
    if (!take(f, v.t + (size_t)ip * v.tt, (size_t)nt)) {
      msg = "truncated table file";
      return JGB_ERR_IO;
    }
    for (int it = 0; it < nt; it++) {
      const size_t r = (size_t)ip * v.tt + it;
      int nu = 0;
      if (!take(f, &nu, 1) || nu < 0) {
        msg = "truncated table file";
        return JGB_ERR_IO;
      }
      if (nu > v.tu) {
        msg = "Too many column densities!";
        return JGB_ERR_ARG;
      }
      v.nu[r] = nu;
      if (!take(f, v.u + r * v.tu, (size_t)nu) || !take(f, v.eps + r * v.tu, (size_t)nu)) {
        msg = "truncated table file";
        return JGB_ERR_IO;
      }
    }
  }
  *np_out = np;
  return JGB_OK;
}

int read_file(const char* path, int fmt, const TblView& v, int* np_out, std::string& msg) {
  FILE* f = std::fopen(path, fmt == 1 ? "r" : "rb");
  if (!f) {
    msg = std::string("cannot open table file ") + path;
    return JGB_ERR_IO;
  }
  clear(v);
  const int rc = fmt == 1 ? read_ascii(f, v, np_out, msg) : read_binary(f, v, np_out, msg);
  std::fclose(f);
  return rc;
}

// ASCII output: a comment header, a blank line before every temperature row
// and one "p T u eps" line per point, with as many digits as reading the
// file back needs to restore every value exactly.
int write_file(const char* path, int fmt, const TblView& v, int np) {
  FILE* f = std::fopen(path, fmt == 1 ? "w" : "wb");
  if (!f) return JGB_ERR_IO;
  bool ok = true;
  if (fmt == 2) {
    ok = std::fwrite(&np, sizeof(int), 1, f) == 1 &&
         std::fwrite(v.p, sizeof(double), (size_t)np, f) == (size_t)np;
    for (int ip = 0; ok && ip < np; ip++) {
      const int nt = v.nt[ip];
      ok = std::fwrite(&nt, sizeof(int), 1, f) == 1 &&
           std::fwrite(v.t + (size_t)ip * v.tt, sizeof(double), (size_t)nt, f) == (size_t)nt;
      for (int it = 0; ok && it < nt; it++) {
        const size_t r = (size_t)ip * v.tt + it;
        const int nu = v.nu[r];
        ok = std::fwrite(&nu, sizeof(int), 1, f) == 1 &&
             std::fwrite(v.u + r * v.tu, sizeof(float), (size_t)nu, f) == (size_t)nu &&
             std::fwrite(v.eps + r * v.tu, sizeof(float), (size_t)nu, f) == (size_t)nu;
      }
    }
  } else {
    ok = std::fputs("# $1 = pressure [hPa]\n# $2 = temperature [K]\n"
                    "# $3 = column density [molecules/cm^2]\n# $4 = emissivity [-]\n",
                    f) >= 0;
    for (int ip = 0; ok && ip < np; ip++)
      for (int it = 0; ok && it < v.nt[ip]; it++) {
        const size_t r = (size_t)ip * v.tt + it;
        ok = std::fputc('\n', f) != EOF;
        for (int iu = 0; ok && iu < v.nu[r]; iu++)
          ok = std::fprintf(f, "%.17g %.17g %.9e %.9e\n", v.p[ip], v.t[r],
                            (double)v.u[r * v.tu + iu], (double)v.eps[r * v.tu + iu]) > 0;
      }
  }
  if (std::fclose(f) != 0) ok = false;
  return ok ? JGB_OK : JGB_ERR_IO;
}

bool valid_caps(int fmt, int tp, int tt, int tu) {
  return (fmt == 1 || fmt == 2) && tp > 0 && tt > 0 && tu > 0;
}

}  // namespace

using namespace jgb;

extern "C" int jgb_read_table_file(const char* path, int tblfmt, int tp, int tt, int tu,
                                   int* np_out, double* p, int* nt, double* t, int* nu, float* u,
                                   float* eps) {
  if (!path || !np_out || !p || !nt || !t || !nu || !u || !eps || !valid_caps(tblfmt, tp, tt, tu))
    return JGB_ERR_ARG;
  std::string msg;
  *np_out = -1;
  return read_file(path, tblfmt, TblView{tp, tt, tu, p, nt, t, nu, u, eps}, np_out, msg);
}

extern "C" int jgb_write_table_file(const char* path, int tblfmt, int np, const double* p,
                                    const int* nt, const double* t, const int* nu, const float* u,
                                    const float* eps, int tt_cap, int tu_cap) {
  if (!path || np < 0 || (np > 0 && (!p || !nt || !t || !nu || !u || !eps)) ||
      !valid_caps(tblfmt, np > 0 ? np : 1, tt_cap, tu_cap))
    return JGB_ERR_ARG;
  for (int ip = 0; ip < np; ip++) {
    if (nt[ip] < 0 || nt[ip] > tt_cap) return JGB_ERR_ARG;
    for (int it = 0; it < nt[ip]; it++) {
      const int n = nu[(size_t)ip * tt_cap + it];
      if (n < 0 || n > tu_cap) return JGB_ERR_ARG;
    }
  }
  const TblView v{np, tt_cap, tu_cap, const_cast<double*>(p), const_cast<int*>(nt),
                  const_cast<double*>(t), const_cast<int*>(nu), const_cast<float*>(u),
                  const_cast<float*>(eps)};
  return write_file(path, tblfmt, v, np);
}

extern "C" int jgb_read_tables(jgb_ctx* x, const char* tblbase, int tblfmt) {
  jgb::CtxLock lock(x);
  if (!x) return JGB_ERR_ARG;
  if (!tblbase || (tblfmt != 1 && tblfmt != 2))
    return ctx_fail(x, JGB_ERR_ARG, "Unknown look-up table format!");
  if (!x->tables_init) return ctx_fail(x, JGB_ERR_STATE, "jgb_tables_init not called");
  const int tp = x->tp, tt = x->tt, tu = x->tu;
  std::vector<double> p(tp), t((size_t)tp * tt);
  std::vector<int> nt(tp), nu((size_t)tp * tt);
  std::vector<float> u((size_t)tp * tt * tu), eps((size_t)tp * tt * tu);
  const TblView v{tp, tt, tu, p.data(), nt.data(), t.data(), nu.data(), u.data(), eps.data()};
  const int nd = (int)x->nu.size(), ng = (int)x->emitter.size();
  for (int id = 0; id < nd; id++)
    for (int ig = 0; ig < ng; ig++) {
      // file name of read_tbl (jurassic.c:4968)
      char fn[4096];
      const int len = std::snprintf(fn, sizeof fn, "%s_%.4f_%s.%s", tblbase, x->nu[id],
                                    x->emitter[ig].c_str(), tblfmt == 1 ? "tab" : "bin");
      if (len < 0 || len >= (int)sizeof fn) return ctx_fail(x, JGB_ERR_ARG, "table file name too long");
      int np = -1;
      FILE* probe = std::fopen(fn, "rb");
      if (probe) {  // a missing file leaves the table empty (the reference warns)
        std::fclose(probe);
        std::string msg;
        const int rc = read_file(fn, tblfmt, v, &np, msg);
        if (rc != JGB_OK) return ctx_fail(x, rc, (msg + " (" + fn + ")").c_str());
      }
      const int rc = jgb_set_table(x, id, ig, np, p.data(), nt.data(), t.data(), nu.data(),
                                   u.data(), eps.data(), tt, tu);
      if (rc != JGB_OK) return rc;
    }
  return JGB_OK;
}
