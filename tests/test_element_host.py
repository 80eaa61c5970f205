"""The element programs of the device kernels, compiled for the host, against the oracle.

The per-cell code the element kernels run (metric, inverse, blade Gramians,
mass/stiffness/coboundary sums) is host+device code; tests/element_host.cu
compiles it with the host compiler, with contraction off, once per (dimension,
arithmetic type). This checks the element algebra and the float-float arithmetic
on CPU at the same tolerances as the GPU parity tests (operators.rs:58-212 via
the oracle's element_matrix).
"""

import concurrent.futures as cf
import ctypes
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "element_host.cu")
CSRC = os.path.join(ROOT, "formoniq_gb300", "csrc")
OUT = os.path.join(ROOT, "tests", "_build")
LIB = os.path.join(OUT, "libelement_host.so")

MASS, DIF_TRIAL, DIF_TEST, DIF_BOTH, HDIF = 0, 1, 2, 3, 4
DF64, F32, F64 = 0, 1, 2
TOL = {DF64: 1e-12, F64: 1e-12, F32: 1e-5}
DIMS = (1, 2, 3, 4)


def _inputs_newer_than(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [SRC] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return any(os.path.getmtime(d) > t for d in deps)


def _build():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    if not _inputs_newer_than(LIB):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = [(t, n) for t in (DF64, F32, F64) for n in DIMS]

    def one(job):
        t, n = job
        obj = os.path.join(OUT, f"element_host_t{t}_n{n}.o")
        cmd = [nvcc, "-std=c++17", "-O1", "--expt-relaxed-constexpr", "-x", "cu", "-Xcompiler",
               "-fPIC,-ffp-contract=off", f"-DEH_TYPE={t}", f"-DEH_DIM={n}", "-I", CSRC, "-c", SRC, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host element build failed ({t}, {n}):\n{r.stderr[-4000:]}")
        return obj

    # the 4D objects take longest: start them first
    jobs.sort(key=lambda j: -j[1])
    with cf.ThreadPoolExecutor(min(len(jobs), max(2, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(one, jobs))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc, "-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host element link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


@pytest.fixture(scope="module")
def host_lib():
    lib = ctypes.CDLL(_build())
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    fns = {}
    for t in (DF64, F32, F64):
        for n in DIMS:
            fn = getattr(lib, f"eh_element_t{t}_n{n}")
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_int, ctypes.c_int, f64p, ctypes.c_double, f64p, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_double)]
            fns[(t, n)] = fn
    return fns


def run(host_lib, t, n, k, kind, lengths, param=0.0):
    out = np.zeros(4096)
    det = ctypes.c_double()
    ne = host_lib[(t, n)](k, kind, np.ascontiguousarray(lengths, np.float64), param, out, out.size,
                          ctypes.byref(det))
    assert ne >= 0, (t, n, k, kind, ne)
    return out[:ne], det.value


def unpack_sym(v, L):
    m = np.zeros((L, L))
    iu = np.triu_indices(L)
    m[iu] = v[: len(iu[0])]
    return m + np.triu(m, 1).T


def rel_frob(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def sample_cells(oracle, dim, seed=3, jitter=0.15):
    cx, coords = oracle.cartesian_unit(dim, 2)
    coords = oracle.jitter_coords(coords, 2, seed, jitter, side=np.ones(dim))
    lengths = cx.edge_lengths_sq(coords)
    edges = cx.cell_faces(1)
    nc = cx.ncells()
    return [lengths[edges[c]] for c in range(0, nc, max(1, nc // 7))]


@pytest.mark.parametrize("dim", DIMS)
@pytest.mark.parametrize("t", [DF64, F32, F64])
def test_whitney_pairings(oracle, host_lib, dim, t):
    for ll in sample_cells(oracle, dim):
        for form in (MASS, DIF_TRIAL, DIF_TEST, DIF_BOTH):
            for grade in range(dim + 1):
                tg = grade - 1 if form in (DIF_TEST, DIF_BOTH) else grade
                sg = grade - 1 if form in (DIF_TRIAL, DIF_BOTH) else grade
                if tg < 0 or sg < 0:
                    continue
                lr, lc = math.comb(dim + 1, tg + 1), math.comb(dim + 1, sg + 1)
                v, _ = run(host_lib, t, dim, grade, form, ll)
                got = unpack_sym(v, lr) if form in (MASS, DIF_BOTH) else v[: lr * lc].reshape(lr, lc)
                expect = oracle.element_matrix(dim, form, grade, ll)
                assert rel_frob(got, expect) < TOL[t], (form, grade)


@pytest.mark.parametrize("dim", DIMS)
@pytest.mark.parametrize("t", [DF64, F64])
def test_hdif_gram(oracle, host_lib, dim, t):
    """hdif_gram(k) = M_k + dif_both(k+1) (whitney_complex.rs:180-183), per cell."""
    for ll in sample_cells(oracle, dim, seed=5):
        for grade in range(dim + 1):
            L = math.comb(dim + 1, grade + 1)
            v, _ = run(host_lib, t, dim, grade, HDIF, ll)
            expect = oracle.element_matrix(dim, MASS, grade, ll)
            if grade + 1 <= dim:
                expect = expect + oracle.element_matrix(dim, DIF_BOTH, grade + 1, ll)
            assert rel_frob(unpack_sym(v, L), expect) < TOL[t], grade


@pytest.mark.parametrize("dim", DIMS)
def test_float_float_beats_float(oracle, host_lib, dim):
    """The float-float programs carry about 48 bits: far below FP32's error."""
    for ll in sample_cells(oracle, dim, seed=9, jitter=0.3):
        for grade in range(1, dim + 1):
            expect = oracle.element_matrix(dim, DIF_BOTH, grade, ll)
            L = expect.shape[0]
            e_df = rel_frob(unpack_sym(run(host_lib, DF64, dim, grade, DIF_BOTH, ll)[0], L), expect)
            e_f = rel_frob(unpack_sym(run(host_lib, F32, dim, grade, DIF_BOTH, ll)[0], L), expect)
            assert e_df < TOL[DF64] and e_df < 1e-4 * e_f, (grade, e_df, e_f)


def test_float_float_conversions_match_rounded_conversions(host_lib):
    """df64(double): the nearest float and the float nearest the exact
    remainder (the conversion instructions' results); to_double: the double
    nearest hi + lo; dd_sqrt: 48-bit square root."""
    lib = ctypes.CDLL(LIB)
    rng = np.random.default_rng(11)
    mant = rng.uniform(1.0, 2.0, 4000)
    expo = rng.integers(-70, 70, 4000).astype(np.float64)
    d = np.concatenate([mant * 2.0 ** expo * rng.choice([-1.0, 1.0], 4000),
                        [0.0, -0.0, 1.0, 3.0, 1e-300, 1e300, 2.0 ** -60, 2.0 ** 60],
                        # ties at the 24-bit boundary: 1 + 2^-24 (round to even) and 1 + 3 2^-24
                        [1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, -(1.0 + 2.0 ** -24), 2.0 - 2.0 ** -53]])
    d = np.ascontiguousarray(d)
    n = len(d)
    hi = np.zeros(n, np.float32)
    lo = np.zeros(n, np.float32)
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    lib.eh_df64_split.argtypes = [f64p, f32p, f32p, ctypes.c_int]
    lib.eh_df64_split(d, hi, lo, n)
    # 1e300 overflows float32 on purpose: its hi is inf and its lo is not compared
    with np.errstate(over="ignore", invalid="ignore"):
        want_hi = d.astype(np.float32)
        want_lo = (d - want_hi.astype(np.float64)).astype(np.float32)
    np.testing.assert_array_equal(hi, want_hi)
    finite = np.isfinite(want_hi)
    np.testing.assert_array_equal(lo[finite], want_lo[finite])
    back = np.zeros(n)
    lib.eh_df64_to_double.argtypes = [f32p, f32p, f64p, ctypes.c_int]
    lib.eh_df64_to_double(hi, lo, back, n)
    with np.errstate(invalid="ignore"):
        want_back = hi.astype(np.float64) + lo.astype(np.float64)
    np.testing.assert_array_equal(back[finite], want_back[finite])
    pos = np.ascontiguousarray(np.abs(d[:4000]))
    ph = pos.astype(np.float32)
    pl = (pos - ph.astype(np.float64)).astype(np.float32)
    sh, sl = np.zeros(4000, np.float32), np.zeros(4000, np.float32)
    lib.eh_df64_sqrt.argtypes = [f32p, f32p, f32p, f32p, ctypes.c_int]
    lib.eh_df64_sqrt(ph, pl, sh, sl, 4000)
    got = sh.astype(np.float64) + sl.astype(np.float64)
    want = np.sqrt(ph.astype(np.float64) + pl.astype(np.float64))
    assert np.max(np.abs(got - want) / want) < 2e-14


@pytest.mark.parametrize("dim", [2, 3, 4])
def test_top_grade_mass_is_the_inverse_volume(oracle, host_lib, dim):
    """The Whitney n-form of an n-cell is 1/vol times its volume form, so its
    mass is exactly 1/vol. The top compound Lambda^n B is formed in closed form
    (+-1/det G), so the float-float program meets this to 1e-13 even on
    strongly distorted cells (0.2h jitter), where the n x n minors of the rank-n
    B -- and the reference's determinant of G^{-1} -- cancel to about 1e-11."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    worst = 0.0
    for seed in range(3):
        c2 = oracle.jitter_coords(coords, 2, seed, 0.2, side=np.ones(dim))
        lengths = cx.edge_lengths_sq(c2)
        edges = cx.cell_faces(1)
        _, _, _, vol, _ = cx.cell_metrics(lengths)
        for c in range(cx.ncells()):
            v, _ = run(host_lib, DF64, dim, dim, 0, lengths[edges[c]])
            worst = max(worst, abs(v[0] * vol[c] - 1.0))
    assert worst < 1e-13, worst
