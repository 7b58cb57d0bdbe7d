"""The C-ABI library loads and exports every entry point include/gbsym.h
declares; the host-only entry points (schedule inspectors, status strings)
run here without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "gbsym.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbsym_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from sympiler_gb300 import _lib
    path = _lib.LIB_PATH
    assert os.path.exists(path), "libgbsym.so not built"
    L = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from sympiler_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == _declared()


def test_library_has_no_cuda_runtime_dependency():
    from sympiler_gb300 import _lib
    out = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "libcudart" not in out


def test_status_strings_without_gpu():
    from sympiler_gb300 import _lib
    L = _lib.lib()
    assert L.gbsym_status_string(0) == b"ok"
    assert b"schedule" in L.gbsym_status_string(_lib.ERR_BAD_SCHEDULE)
    assert L.gbsym_last_error() == 0


def test_cpp_shim_compiles_and_links(tmp_path):
    """A caller written against the reference's sym_lib signatures compiles
    against include/gbsym_sym_lib.hpp and links libgbsym.so (nothing is run:
    no GPU here)."""
    from sympiler_gb300 import _lib
    src = tmp_path / "caller.cpp"
    src.write_text(r'''
#include "gbsym_sym_lib.hpp"
#include <cstdio>
int main(int argc, char **argv) {
  if (argc > 99) {  // never taken: only the symbols and signatures matter here
    int n = 1, p[2] = {0, 1}, i[1] = {0}, *lp = nullptr, *ls = nullptr;
    double v[1] = {1.0}, x[1] = {1.0}, y[1] = {0.0}, z[1] = {0.0};
    sym_lib::sptrsv_csr(n, p, i, v, x);
    sym_lib::sptrsv_csr_levelset(n, p, i, v, x, 1, p, i);
    sym_lib::sptrsv_csr_lbc(n, p, i, v, x, 1, p, p, i);
    sym_lib::sptrsv_csr_ilu(n, p, i, v, i, x);
    sym_lib::sptrsv_csc(n, p, i, v, x);
    sym_lib::spmv_csr(n, p, i, v, x, y);
    sym_lib::spmv_csr(n, p, i, v, x, y, z, 1.0, 0.0);
    sym_lib::ltsolve(n, p, i, v, x);
    sym_lib::spic0_csr(n, v, p, i);
    sym_lib::spic0_csr_lbc(n, v, p, i, 1, p, p, i);
    sym_lib::spilu0_csr(n, 1, p, i, v, i, y);
    sym_lib::spilu0_csr_lbc(n, 1, p, i, v, i, y, 1, p, p, i, nullptr);
    sym_lib::parsy::lsolve(n, p, i, v, x);
    sym_lib::parsy::lus_cr(n, 1, p, i, v, i, x, y);
    size_t zp[2] = {0, 1};
    sym_lib::parsy::blockedLsolve(n, zp, i, v, 1, zp, i, p, 1, x);
    sym_lib::parsy::H2LeveledBlockedLTsolve(n, zp, i, v, 1, zp, i, p, 1, x, 1, p, i, 1, p, i, 1);
    sym_lib::parsy::solve_phase_ll_blocked(1, x, i, p, zp, i, v, zp, 1, 1);
    sym_lib::parsy::solve_phase_ldl(1, v, x, i, p, zp, i, v, zp, 1, 1);
    sym_lib::parsy::solve_phase_simplicial_ll(n, p, i, v, x);
    sym_lib::parsy::solve_phase_simplicial_ldl(n, p, i, v, v, x);
    sym_lib::build_levelSet_CSC(1, p, i, lp, ls);
    delete[] lp; delete[] ls;
  }
  std::printf("%s\n", gbsym_status_string(gbsym_last_error()));
  return 0;
}
''')
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L" + libdir, "-lgbsym", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out


def test_cpp_shim_runs_lbc_inspectors(tmp_path):
    """The inspectors are host code: a C++ caller of the reference's
    signatures runs them here and gets what the Python binding gets."""
    from sympiler_gb300 import _lib, sym_lib
    from sympiler_gb300 import matgen as mg
    L = mg.tril(mg.random_spd(300, 3, np.random.default_rng(4)))
    src = tmp_path / "inspect.cpp"
    arr = lambda a: ",".join(str(int(v)) for v in a)  # noqa: E731
    src.write_text(r'''
#include "gbsym_sym_lib.hpp"
#include <cstdio>
static const int Lp[] = {%s};
static const int Li[] = {%s};
int main() {
  const int n = %d;
  int nl = 0, np = 0, *lp = nullptr, *pp = nullptr, *nd = nullptr;
  double *cost = nullptr;
  sym_lib::get_coarse_levelSet_DAG_CSC_tree(n, Lp, Li, 0, nl, lp, np, pp, nd, 4, -1, 100, cost);
  std::printf("%%d %%d\n", nl, np);
  for (int i = 0; i <= nl; ++i) std::printf("%%d ", lp[i]);
  std::printf("\n");
  for (int i = 0; i <= np; ++i) std::printf("%%d ", pp[i]);
  std::printf("\n");
  for (int i = 0; i < n; ++i) std::printf("%%d ", nd[i]);
  std::printf("\n");
  delete[] lp; delete[] pp; delete[] nd;
  int parent[n], tlp[n + 1], tls[n];
  gbsym_etree_lower_csr(n, Lp, Li, parent);
  std::printf("%%d\n", sym_lib::parsy::getLevelSet(n, parent, tlp, tls));
  return 0;
}
''' % (arr(L.p), arr(L.i), L.n))
    exe = tmp_path / "inspect"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L" + libdir, "-lgbsym", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.split("\n")
    nl, lp, pn, pp, nodes = sym_lib.get_coarse_levelSet_DAG_CSC_tree(L.n, L.p, L.i, 0, 4, -1, 100)
    assert lines[0].split() == [str(nl), str(pn)]
    assert [int(v) for v in lines[1].split()] == list(lp)
    assert [int(v) for v in lines[2].split()] == list(pp)
    assert [int(v) for v in lines[3].split()] == list(nodes)
    par = sym_lib.etree_lower_csr(L.n, L.p, L.i)
    tlp, tls = np.zeros(L.n + 1, np.int32), np.zeros(L.n, np.int32)
    assert int(lines[4]) == sym_lib.parsy.getLevelSet(L.n, par, tlp, tls)


def test_lbc_factor_drop_ins_check_arguments_on_the_host():
    """spilu0_csr_lbc / spic0_csr_lbc report argument errors before any
    device work, so these run without a GPU: n = 0 is a no-op, null arrays
    give NULL_ARG, and an upper CSR whose row does not start with its
    diagonal gives BAD_MATRIX under an LBC schedule."""
    import ctypes as C
    from sympiler_gb300 import _lib
    L = _lib.lib()
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    L.gbsym_spilu0_csr_lbc(0, 0, None, None, None, None, None, 0, None, None, None, None)
    assert L.gbsym_last_error() == _lib.OK
    L.gbsym_spic0_csr_lbc(0, None, None, None, 0, None, None, None)
    assert L.gbsym_last_error() == _lib.OK
    L.gbsym_spilu0_csr_lbc(3, 3, None, None, None, None, None, 1, None, None, None, None)
    assert L.gbsym_last_error() == _lib.ERR_NULL_ARG
    L.gbsym_spic0_csr_lbc(3, None, None, None, 1, None, None, None)
    assert L.gbsym_last_error() == _lib.ERR_NULL_ARG
    rp = np.array([0, 2, 3, 4], np.int32)
    ci = np.array([0, 2, 2, 2], np.int32)  # row 1 starts with column 2, not its diagonal
    v = np.ones(4)
    lp, pp, part = np.array([0, 1], np.int32), np.array([0, 3], np.int32), np.arange(3, dtype=np.int32)
    L.gbsym_spic0_csr_lbc(3, P(v), P(rp), P(ci), 1, P(lp), P(pp), P(part))
    assert L.gbsym_last_error() == _lib.ERR_BAD_MATRIX
    assert np.all(v == 1.0)


@pytest.mark.parametrize("name,nint", [("gbsym_sptrsv_csr", 0), ("gbsym_sptrsv_csc", 0), ("gbsym_spmv_csr", 0),
                                       ("gbsym_spilu0_csr", 1), ("gbsym_parsy_lus_cr", 1),
                                       ("gbsym_sptrsv_csr_levelset", 0)])
def test_drop_ins_report_null_arrays_without_a_gpu(name, nint):
    """The void drop-ins record NULL_ARG for null arrays, and n = 0 is a
    no-op, before any device work (so these run without a GPU); the int
    forms also return 0."""
    from sympiler_gb300 import _lib
    L = _lib.lib()
    f = getattr(L, name)
    argtypes = _lib.SIGNATURES[name][1]
    def args(n):
        out = [n]
        ints_left = nint
        for t in argtypes[1:]:
            if t is _lib.C.c_int:
                out.append(n if ints_left else 1)
                ints_left = max(0, ints_left - 1)
            else:
                out.append(None)
        return out
    f(*args(0))
    assert L.gbsym_last_error() == _lib.OK
    f(*args(4))
    assert L.gbsym_last_error() == _lib.ERR_NULL_ARG
    for fn in (L.gbsym_ltsolve, L.gbsym_parsy_lsolve):
        assert fn(4, None, None, None, None) == 0
        assert L.gbsym_last_error() == _lib.ERR_NULL_ARG


@pytest.mark.gpu
def test_cpp_shim_runs_on_the_gpu(gpu, tmp_path):
    """A caller written against the reference's sym_lib signatures, compiled
    against include/gbsym_sym_lib.hpp and linked to libgbsym.so, solves on
    the GPU: sptrsv_csr, sptrsv_csr_levelset with the level set from
    build_levelSet_CSC, sptrsv_csc, ltsolve and spmv_csr on a 2D Laplacian,
    each compared bit for bit inside the program with a plain serial loop in
    the reference's operation order (compiled without contraction)."""
    from sympiler_gb300 import _lib
    src = tmp_path / "gpu_caller.cpp"
    src.write_text(r'''
#include "gbsym_sym_lib.hpp"
#include <cstdio>
#include <cstring>
#include <vector>
int main() {
  const int g = 60, n = g * g;
  std::vector<int> Lp(n + 1), Li;          // lower CSR of the 5-point Laplacian, diagonal last
  std::vector<double> Lx;
  std::vector<int> Ap(n + 1), Ai;          // full CSR
  std::vector<double> Ax;
  for (int i = 0; i < n; ++i) {
    const int x = i % g, y = i / g;
    if (y > 0) { Li.push_back(i - g); Lx.push_back(-1.0); }
    if (x > 0) { Li.push_back(i - 1); Lx.push_back(-1.0); }
    Li.push_back(i); Lx.push_back(4.0 + 0.01 * (i % 7));
    Lp[i + 1] = (int)Li.size();
    if (y > 0) { Ai.push_back(i - g); Ax.push_back(-1.0); }
    if (x > 0) { Ai.push_back(i - 1); Ax.push_back(-1.0); }
    Ai.push_back(i); Ax.push_back(4.0 + 0.01 * (i % 7));
    if (x < g - 1) { Ai.push_back(i + 1); Ax.push_back(-1.0); }
    if (y < g - 1) { Ai.push_back(i + g); Ax.push_back(-1.0); }
    Ap[i + 1] = (int)Ai.size();
  }
  // CSC of L (diagonal first in each column) = upper CSR of L^T
  std::vector<int> Cp(n + 1, 0), Ci(Li.size());
  std::vector<double> Cx(Li.size());
  for (int e = 0; e < (int)Li.size(); ++e) Cp[Li[e] + 1]++;
  for (int j = 0; j < n; ++j) Cp[j + 1] += Cp[j];
  std::vector<int> fill(Cp.begin(), Cp.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int e = Lp[i]; e < Lp[i + 1]; ++e) { Ci[fill[Li[e]]] = i; Cx[fill[Li[e]]++] = Lx[e]; }
  std::vector<double> b(n);
  for (int i = 0; i < n; ++i) b[i] = ((i * 37) % 101) / 50.0 - 1.0;
  // serial checks in the reference's order
  std::vector<double> want(b);
  for (int i = 0; i < n; ++i) {
    double xi = want[i];
    for (int e = Lp[i]; e < Lp[i + 1] - 1; ++e) xi -= Lx[e] * want[Li[e]];
    want[i] = xi / Lx[Lp[i + 1] - 1];
  }
  std::vector<double> want_t(b);           // L^T x = b on the CSC of L
  for (int j = n - 1; j >= 0; --j) {
    double xj = want_t[j];
    for (int e = Cp[j] + 1; e < Cp[j + 1]; ++e) xj -= Cx[e] * want_t[Ci[e]];
    want_t[j] = xj / Cx[Cp[j]];
  }
  std::vector<double> want_y(n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int e = Ap[i]; e < Ap[i + 1]; ++e) want_y[i] += Ax[e] * b[Ai[e]];
  int bad = 0;
  auto same = [&](const std::vector<double> &a, const std::vector<double> &c, const char *what) {
    if (std::memcmp(a.data(), c.data(), a.size() * sizeof(double)) != 0) {
      std::printf("%s differs\n", what);
      ++bad;
    }
  };
  std::vector<double> x(b);
  sym_lib::sptrsv_csr(n, Lp.data(), Li.data(), Lx.data(), x.data());
  same(x, want, "sptrsv_csr");
  int *lptr = nullptr, *lset = nullptr;
  const int levels = sym_lib::build_levelSet_CSC(n, Cp.data(), Ci.data(), lptr, lset);
  x = b;
  sym_lib::sptrsv_csr_levelset(n, Lp.data(), Li.data(), Lx.data(), x.data(), levels, lptr, lset);
  same(x, want, "sptrsv_csr_levelset");
  delete[] lptr;
  delete[] lset;
  x = b;
  sym_lib::sptrsv_csc(n, Cp.data(), Ci.data(), Cx.data(), x.data());
  same(x, want, "sptrsv_csc");
  x = b;
  if (sym_lib::ltsolve(n, Cp.data(), Ci.data(), Cx.data(), x.data()) != 1) ++bad;
  same(x, want_t, "ltsolve");
  std::vector<double> y(n, 0.0);
  sym_lib::spmv_csr(n, Ap.data(), Ai.data(), Ax.data(), b.data(), y.data());
  same(y, want_y, "spmv_csr");
  std::printf("%s levels=%d\n", bad ? "FAILED" : "ok", levels);
  return bad || gbsym_last_error() != 0;
}
''')
    exe = tmp_path / "gpu_caller"
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++11", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe), "-L" + libdir, "-lgbsym", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("ok levels=119"), (out.stdout, out.stderr)
