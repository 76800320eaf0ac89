"""GPU parity of calcTCC (litho.cpp:428-516) and calcKernels (litho.cpp:579-645).

Kernels are compared up to phase and within degenerate eigen-subspaces: for each
cluster of (near-)equal eigenvalues the orthogonal projector V V^H is compared,
which is invariant to the basis the eigensolver picks inside the cluster.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import np_ref as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    import litho_gb300
    return litho_gb300


@pytest.fixture(scope="module")
def ctx(L):
    c = L.Context(0)
    yield c
    c.close()


def _clusters(w, rel=1e-6):
    groups, cur = [], [0]
    for i in range(1, len(w)):
        if abs(w[i - 1] - w[i]) <= rel * max(abs(w[0]), 1e-300):
            cur.append(i)
        else:
            groups.append(cur)
            cur = [i]
    groups.append(cur)
    return groups


def _compare_kernels(krn_gpu, s_gpu, krn_ref, s_ref, w_all, tol_vec=1e-8):
    """w_all: the full descending spectrum, used to skip a cluster that nk cuts
    (its kept vector is an arbitrary member of a larger eigenspace)."""
    np.testing.assert_allclose(s_gpu, s_ref, rtol=1e-11, atol=1e-13 * abs(s_ref[0]))
    nk = len(s_ref)
    for g in _clusters(np.asarray(w_all)):
        if g[0] >= nk:
            break
        if g[-1] >= nk:
            continue
        A = krn_gpu[g].T
        B = krn_ref[g].T
        Pa = A @ A.conj().T
        Pb = B @ B.conj().T
        assert np.linalg.norm(Pa - Pb) < tol_vec * len(g), (g, np.linalg.norm(Pa - Pb))


def test_tcc_fp64_matches_reference_golden(ctx, golden_optics):
    g = golden_optics
    tcc = ctx.calc_tcc(g["src"], g["sigma"], 193.0, 0.8, 0.2, 512, 512, g["Nx"], g["Nx"])
    ref = load_golden("tcc_golden.npz")
    gold = ref["tcc_r"].astype(np.float64) + 1j * ref["tcc_i"].astype(np.float64)
    assert np.linalg.norm(tcc - gold) / np.linalg.norm(gold) < 1e-7
    assert np.linalg.norm(tcc - g["tcc"]) / np.linalg.norm(g["tcc"]) < 1e-7
    assert np.array_equal(tcc, tcc.conj().T)


@pytest.mark.parametrize("case", ["annular21_512", "quasar_1024", "annular101_defocus"])
def test_tcc_fp64_matches_oracle(ctx, case):
    from litho_gb300 import synth
    if case == "annular21_512":
        src, L_, df = synth.annular_source(21, 0.6, 0.9), 512, 0.0
    elif case == "quasar_1024":
        src, L_, df = synth.quasar_source(2000)[0], 1024, 0.0
    else:
        src, L_, df = synth.annular_source(101, 0.5, 0.8), 256, 0.3
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, L_, sig, 193.0)
    ref = R.calc_tcc(src, sig, 193.0, 0.8, df, L_, L_, nx, nx)
    tcc = ctx.calc_tcc(src, sig, 193.0, 0.8, df, L_, L_, nx, nx)
    assert np.linalg.norm(tcc - ref) / np.linalg.norm(ref) < 1e-7


def test_kernels_match_oracle_golden(ctx, golden_optics, L):
    g = golden_optics
    k_gpu, s32, s64 = ctx.calc_kernels(g["tcc"], 10)
    k_ref, s_ref32, w_ref = R.calc_kernels(g["tcc"], 10)
    np.testing.assert_allclose(s32, load_golden("tcc_golden.npz")["eigenvalues"], rtol=6e-6)
    _compare_kernels(k_gpu, s64, k_ref, w_ref, np.linalg.eigvalsh(g["tcc"])[::-1])
    # unit norm, mutually orthogonal
    G = k_gpu @ k_gpu.conj().T
    assert np.abs(G - np.eye(10)).max() < 1e-12


def test_kernels_are_eigenvectors_reversed(ctx, golden_optics):
    """krn[i][j] = v_i[n-1-j] (litho.cpp:626-634): T v = lambda v with v = krn reversed."""
    tcc = golden_optics["tcc"]
    k_gpu, _, s64 = ctx.calc_kernels(tcc, 81)
    for i in range(81):
        v = k_gpu[i][::-1]
        assert np.linalg.norm(tcc @ v - s64[i] * v) < 1e-11 * abs(s64[0])
    assert np.all(np.diff(s64) <= 0)


def test_kernels_config2_quasar(ctx):
    from litho_gb300 import synth
    src = synth.quasar_source(2000)[0]
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, 1024, sig, 193.0)
    tcc = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, 1024, 1024, nx, nx)
    k_gpu, _, s64 = ctx.calc_kernels(tcc, 24)
    w = np.linalg.eigvalsh(tcc)[::-1]
    # the 24-th eigenvalue must not be split from a partner beyond the cut
    assert abs(w[23] - w[24]) > 1e-6 * w[0]
    k_ref, _, w_ref = R.calc_kernels(tcc, 24)
    _compare_kernels(k_gpu, s64, k_ref, w_ref, w)


def test_full_path_tcc_kernels_image(ctx):
    """GPU TCC -> GPU kernels -> GPU image vs the oracle's full path (config-1 optics)."""
    from litho_gb300 import synth
    mask = synth.rect_mask(512, 40, 8, 64, seed=1)
    src = synth.annular_source(21, 0.6, 0.9)
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, 512, sig, 193.0)
    tcc = ctx.calc_tcc(src, sig, 193.0, 0.8, 0.2, 512, 512, nx, nx)
    krn, s32, _ = ctx.calc_kernels(tcc, 10)
    img = ctx.image(mask, krn, s32, nx, nx)
    tcc_r = R.calc_tcc(src, sig, 193.0, 0.8, 0.2, 512, 512, nx, nx)
    kr, sr, _ = R.calc_kernels(tcc_r, 10)
    ref = R.mask_to_image(mask, kr, sr, nx, nx)
    assert R.rel_l2(img, ref) < 1e-5


@pytest.mark.parametrize("case", ["annular21_512", "quasar_1024"])
def test_tcc_split_bf16_close_to_fp64(ctx, L, case):
    """Three-term BF16 split products with FP32 accumulation (tcgen05): ~1e-5 relative."""
    from litho_gb300 import synth
    src, L_ = (synth.annular_source(21, 0.6, 0.9), 512) if case == "annular21_512" else \
        (synth.quasar_source(2000)[0], 1024)
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, L_, sig, 193.0)
    ref = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, L_, L_, nx, nx)
    tcc = ctx.calc_tcc(src, sig, 193.0, 0.8, 0.0, L_, L_, nx, nx, precision=L.TCC_SPLIT_BF16)
    err = np.linalg.norm(tcc - ref) / np.linalg.norm(ref)
    assert err < 5e-5, err
    assert np.array_equal(tcc, tcc.conj().T)


@pytest.mark.parametrize("shape", [(64, 64), (128, 64), (256, 64), (128, 32), (256, 32)])
@pytest.mark.parametrize("sched", [0, 1, 2])
@pytest.mark.parametrize("case", ["annular21_512", "quasar_1024"])
def test_tcc_split_bf16_every_gemm_shape(ctx, L, case, shape, sched):
    """Every shape the GEMM autotuner may pick (column tile width, K slice, schedule) gives the
    split-BF16 TCC within the same bar, at tcc 81 and 289 (fewer tiles than SMs: the K-split
    schedules spread one tile over many CTAs and sum their partial slots)."""
    from litho_gb300 import synth
    src, L_ = (synth.annular_source(21, 0.6, 0.9), 512) if case == "annular21_512" else \
        (synth.quasar_source(2000)[0], 1024)
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, L_, sig, 193.0)
    ref = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, L_, L_, nx, nx)
    ctx.tcc_gemm_shape(shape[0], shape[1], sched)
    try:
        tcc = ctx.calc_tcc(src, sig, 193.0, 0.8, 0.0, L_, L_, nx, nx, precision=L.TCC_SPLIT_BF16)
        again = ctx.calc_tcc(src, sig, 193.0, 0.8, 0.0, L_, L_, nx, nx, precision=L.TCC_SPLIT_BF16)
    finally:
        ctx.tcc_gemm_shape(0)
    err = np.linalg.norm(tcc - ref) / np.linalg.norm(ref)
    assert err < 5e-5, err
    assert np.array_equal(tcc, tcc.conj().T)
    assert np.array_equal(tcc, again)  # fixed summation order: reproducible


def test_tcc_gemm_shape_rejects_bad_width(ctx, L):
    for bn, bk, sched in ((96, 64, 0), (64, 32, 0), (128, 16, 0), (128, 64, 3)):
        with pytest.raises(L.LithoError) as e:
            ctx.tcc_gemm_shape(bn, bk, sched)
        assert e.value.status == L.LITHO_ERR_ARG


def test_mixed_chain_config2_vs_fp64(ctx, L):
    """Split-BF16 TCC -> FP64 eigensolve -> split-TF32 imaging, vs the all-FP64 oracle: <= 1e-4."""
    from litho_gb300 import synth
    src = synth.quasar_source(2000)[0]
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, 1024, sig, 193.0)
    tcc = ctx.calc_tcc(src, sig, 193.0, 0.8, 0.0, 1024, 1024, nx, nx, precision=L.TCC_SPLIT_BF16)
    krn, s32, _ = ctx.calc_kernels(tcc, 24)
    mask = synth.manhattan_mask(1024, seed=77)
    ks = ctx.kernel_set(krn, s32, nx, nx)
    img = ctx.image_batch(ks, mask[None], precision=L.PREC_MIXED)[0]
    ks.close()
    tcc_r = R.calc_tcc(src, sig, 193.0, 0.8, 0.0, 1024, 1024, nx, nx)
    kr, sr, _ = R.calc_kernels(tcc_r, 24)
    ref = R.mask_to_image(mask, kr, sr, nx, nx)
    assert R.rel_l2(img, ref) < 1e-4


def test_tcc_and_kernel_errors(ctx, golden_optics, L):
    g = golden_optics
    with pytest.raises(L.LithoError) as e:   # Nx too small for the pupil support
        ctx.calc_tcc(g["src"], g["sigma"], 193.0, 0.8, 0.2, 512, 512, 2, 2)
    assert e.value.status == L.LITHO_ERR_ARG
    with pytest.raises(L.LithoError) as e:
        ctx.calc_kernels(g["tcc"], 82)
    assert e.value.status == L.LITHO_ERR_ARG
