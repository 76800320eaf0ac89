"""The large-TCC workload: 2048 x 2048 period at 1 nm/px, NA 1.35 (immersion), 193 nm,
annular source sigma 0.7-0.95 on a 113 x 113 grid (4,044 lit points).  The
reference's Nx formula gives Nx = 27, a 3025 x 3025 TCC, and its pupil phase is
NaN for NA > 1 (litho.cpp:463); the immersion form with n = 1.44 (water at
193 nm) is used.  GPU split-BF16 and FP64 TCCs are checked against the numpy
FP64 restatement, and the GPU FP64 eigensolver's top 48 eigenpairs against
LAPACK (scipy, subset of the spectrum)."""
import time

import numpy as np
import pytest

from oracle import np_ref as R

pytestmark = pytest.mark.gpu

NA, LAM, L, NMED, K = 1.35, 193.0, 2048, 1.44, 48


@pytest.fixture(scope="module")
def setup():
    import litho_gb300 as LG
    from litho_gb300 import synth
    src = synth.annular_source(113, 0.7, 0.95)
    sig = LG.outer_sigma(src)
    nx = LG.optics_n(NA, L, sig, LAM)
    ctx = LG.Context(0)
    t0 = time.time()
    ref = R.calc_tcc(src, sig, LAM, NA, 0.0, L, L, nx, nx, n_medium=NMED)
    t_ref = time.time() - t0
    yield dict(ctx=ctx, LG=LG, src=src, sig=sig, nx=nx, ref=ref, t_ref=t_ref)
    ctx.close()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_reference_formula_is_nan_at_na_above_one(setup):
    LG, ctx = setup["LG"], setup["ctx"]
    with pytest.raises(LG.LithoError) as e:
        ctx.calc_tcc(setup["src"], setup["sig"], LAM, NA, 0.0, L, L, setup["nx"], setup["nx"])
    assert e.value.status == LG.LITHO_ERR_NAN


def test_tcc_3025(setup):
    LG, ctx, ref, nx = setup["LG"], setup["ctx"], setup["ref"], setup["nx"]
    assert nx == 27 and ref.shape == (3025, 3025)
    t0 = time.time()
    t64 = ctx.calc_tcc(setup["src"], setup["sig"], LAM, NA, 0.0, L, L, nx, nx, precision=LG.TCC_FP64, n_medium=NMED)
    t1 = time.time()
    tbf = ctx.calc_tcc(setup["src"], setup["sig"], LAM, NA, 0.0, L, L, nx, nx, precision=LG.TCC_SPLIT_BF16,
                       n_medium=NMED)
    t2 = time.time()
    e64, ebf = _rel(t64, ref), _rel(tbf, ref)
    print(f"tcc 3025: FP64 {t1 - t0:.3f} s rel {e64:.2e}; split-BF16 {t2 - t1:.3f} s rel {ebf:.2e}; "
          f"numpy {setup['t_ref']:.1f} s")
    assert np.isfinite(t64).all() and e64 < 1e-9
    assert ebf < 5e-5
    setup["t64"], setup["tbf"] = t64, tbf


SHAPES = [(64, 64), (128, 64), (256, 64), (128, 32), (256, 32)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("sched", [0, 1, 2])
def test_tcc_3025_every_gemm_shape(setup, shape, sched):
    """Every candidate the GEMM autotuner may pick gives the same split-BF16 TCC."""
    LG, ctx, ref, nx = setup["LG"], setup["ctx"], setup["ref"], setup["nx"]
    ctx.tcc_gemm_shape(shape[0], shape[1], sched)
    try:
        tbf = ctx.calc_tcc(setup["src"], setup["sig"], LAM, NA, 0.0, L, L, nx, nx, precision=LG.TCC_SPLIT_BF16,
                           n_medium=NMED)
    finally:
        ctx.tcc_gemm_shape(0)
    assert _rel(tbf, ref) < 5e-5
    assert np.array_equal(tbf, tbf.conj().T)


def test_tcc_3025_tuning_record(setup):
    tun = [t for t in setup["ctx"].tcc_gemm_tuning() if t["n"] == 3025]
    assert len(tun) == 1
    t = tun[0]
    assert len(t["candidates"]) == 3 * len(SHAPES)
    best = min(t["candidates"], key=lambda c: c["ms"])
    assert (best["bn"], best["bk"], best["sched"]) == (t["bn"], t["bk"], t["sched"])
    print("tcc 3025 GEMM tuning:", t)


def test_top48_eigenpairs(setup):
    from scipy.linalg import eigh
    ctx, ref = setup["ctx"], setup["ref"]
    n = ref.shape[0]
    t0 = time.time()
    w, v = eigh(ref, subset_by_index=[n - K - 1, n - 1], driver="evr")  # K + 1: see whether K cuts a cluster
    t_cpu = time.time() - t0
    w, v = w[::-1], v[:, ::-1]
    for form in ("t64", "tbf"):
        T = setup[form]
        t0 = time.time()
        k64, s32, s64 = ctx.calc_kernels(T, K)
        t_gpu = time.time() - t0
        ew = float(np.max(np.abs(s64 - w[:K]) / np.abs(w[:K])))
        V = k64[:, ::-1].T  # kernels are eigenvectors stored reversed (litho.cpp:632)
        proj, i = 0.0, 0
        while i < K:
            j = i + 1
            while j <= K and abs(w[j - 1] - w[j]) <= 1e-6 * w[0]:
                j += 1
            if j <= K:  # cluster [i, j) lies inside the kept set
                a, b = V[:, i:j], v[:, i:j]
                proj = max(proj, float(np.linalg.norm(a @ a.conj().T - b @ b.conj().T)))
            i = j
        print(f"{form}: GPU eigensolve (n=3025, K=48) {t_gpu:.3f} s; LAPACK subset {t_cpu:.1f} s; "
              f"max eigenvalue rel err {ew:.2e}; max projector err {proj:.2e}")
        if form == "t64":
            assert ew < 1e-9 and proj < 1e-6
        else:
            assert ew < 1e-4 and proj < 1e-2
