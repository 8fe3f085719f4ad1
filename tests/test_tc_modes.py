"""The tensor-core product kernel of the LU (k_tc_update: tcgen05 TF32 MMAs,
FP32 accumulation in TMEM, TMA reduce-add or store epilogue) in every tile mode
it runs, against an exact numpy product of the same operands.

The operands hold TF32 values (10-bit mantissas), so each real product is exact
in FP32 and the only errors are the FP32 accumulation over the 2K real terms of
a complex product (K = 128 or 256), the reduce-add into C, and, in the modes that
store rounded operands, one rounding to TF32.  The bound per element is
    |got - exact| <= 4 (2K + 2) 2^-24 (|C| + sum_k |a_k| |b_k|) [+ 2^-11 |exact|]
i.e. about K 2^-24 relative, far tighter than a TF32-vs-FP32 comparison."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U24 = 2.0 ** -24


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


def tf32(x):
    """Round FP32 values to TF32 (nearest, ties away), as cvt.rna.tf32.f32 does."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x1000) & 0xFFFFE000).astype(np.uint32)
    return b.view(np.float32).astype(np.float64)


def crand(rng, *shape, scale=1.0):
    return tf32(scale * rng.standard_normal(shape)) + 1j * tf32(scale * rng.standard_normal(shape))


def as32(z):
    """The complex value the kernel sees after the FP32 planar copy."""
    return np.asarray(z.real, np.float32).astype(np.float64) + 1j * np.asarray(z.imag, np.float32).astype(np.float64)


def mag(a, b):
    """Elementwise sum_k |a_ik| |b_jk| for real and imaginary outputs of a b^T (each
    output is a sum of 2K real products)."""
    ar, ai, br, bi = np.abs(a.real), np.abs(a.imag), np.abs(b.real), np.abs(b.imag)
    return ar @ br.T + ai @ bi.T, ar @ bi.T + ai @ br.T


def check(got, exact, c0, m_re, m_im, K, rounded=False):
    tol_re = 4 * (2 * K + 2) * U24 * (np.abs(c0.real) + m_re)
    tol_im = 4 * (2 * K + 2) * U24 * (np.abs(c0.imag) + m_im)
    if rounded:
        tol_re = tol_re + 2.0 ** -11 * np.abs(exact.real)
        tol_im = tol_im + 2.0 ** -11 * np.abs(exact.imag)
    er, ei = np.abs(got.real - exact.real), np.abs(got.imag - exact.imag)
    scale = K * U24 * (np.abs(c0) + np.hypot(m_re, m_im)).max()
    print("max err %.3e = %.2f x K 2^-24 x max|C|+sum|a||b|" % (max(er.max(), ei.max()),
                                                                  max(er.max(), ei.max()) / scale))
    assert np.all(er <= tol_re) and np.all(ei <= tol_im), (float((er / tol_re).max()), float((ei / tol_im).max()))


@pytest.mark.parametrize("n", [512, 1024])
def test_trailing_update_modes(bg, n):
    rng = np.random.default_rng(n)
    C = as32(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    Wa, Ua, Wb, Ub = (crand(rng, n, 128, scale=0.2) for _ in range(4))
    m = n - 128
    # mode 0: one step, K = 128
    got, _ = bg.tc_probe(0, C, Wa, Ua)
    exact = C.copy()
    exact[128:, 128:] -= Wa[:m] @ Ua[:m].T
    mr, mi = mag(Wa[:m], Ua[:m])
    check(got[128:, 128:], exact[128:, 128:], C[128:, 128:], mr, mi, 128)
    assert np.array_equal(got[:128], C[:128]) and np.array_equal(got[:, :128], C[:, :128])
    # mode 1: two steps in one pass, K = 256
    got, _ = bg.tc_probe(1, C, Wa, Ua, Wb, Ub)
    exact = C.copy()
    exact[128:, 128:] -= Wa[:m] @ Ua[:m].T + Wb[:m] @ Ub[:m].T
    mr2, mi2 = mag(Wb[:m], Ub[:m])
    check(got[128:, 128:], exact[128:, 128:], C[128:, 128:], mr + mr2, mi + mi2, 256)
    # mode 2: only the L of width 2 (tile columns 0-1, then tile rows 0-1), first tile dropped
    got, _ = bg.tc_probe(2, C, Wa, Ua, Wb, Ub)
    mask = np.zeros((m, m), bool)
    mask[:, :256] = True
    mask[:256, :] = True
    mask[:128, :128] = False
    sub = got[128:, 128:]
    check(sub[mask], exact[128:, 128:][mask], C[128:, 128:][mask], (mr + mr2)[mask], (mi + mi2)[mask], 256)
    assert np.array_equal(sub[~mask], C[128:, 128:][~mask])


@pytest.mark.parametrize("n", [512, 1024])
def test_w21_and_u_column_modes(bg, n):
    rng = np.random.default_rng(7 + n)
    C = crand(rng, n, n)
    Dinv = crand(rng, 128, 128, scale=0.1)  # the block inverse; the kernel takes its transpose
    T = Dinv.T.copy()
    # mode 3: W21 = A21 D^-1, stored rounded into W and over A21
    got, W = bg.tc_probe(3, C, T=T)
    exact = C[128:, :128] @ Dinv
    mr, mi = mag(C[128:, :128], T)
    check(W[:n - 128], exact, 0 * exact, mr, mi, 128, rounded=True)
    assert np.array_equal(got[128:, :128], W[:n - 128])
    assert np.array_equal(got[:128], C[:128]) and np.array_equal(got[128:, 128:], C[128:, 128:])
    # mode 4: the last column block of U times D^-1, rounded, in place
    got, _ = bg.tc_probe(4, C, T=T)
    exact = C[:n - 128, n - 128:] @ Dinv
    mr, mi = mag(C[:n - 128, n - 128:], T)
    check(got[:n - 128, n - 128:], exact, 0 * exact, mr, mi, 128, rounded=True)
    assert np.array_equal(got[:, :n - 128], C[:, :n - 128]) and np.array_equal(got[n - 128:], C[n - 128:])


@pytest.mark.parametrize("n", [512, 1024])
def test_pair_fold_modes(bg, n):
    rng = np.random.default_rng(11 + n)
    C = crand(rng, n, n)
    nb, npair = n // 128, n // 256
    T = crand(rng, npair, 128, 128, scale=0.1)
    blk = lambda M, r, c: M[128 * r:128 * (r + 1), 128 * c:128 * (c + 1)]
    for mode, which in ((5, 1), (6, 2)):
        got, _ = bg.tc_probe(mode, C, T=T)
        exact = C.copy()
        touched = np.zeros((nb, nb), bool)
        for p in range(npair):
            rows = range(2 * p + 2, nb) if which == 1 else range(0, 2 * p)
            for r in rows:
                src, dst = (2 * p + 1, 2 * p) if which == 1 else (2 * p, 2 * p + 1)
                prod = blk(C, r, src) @ T[p].T
                blk(exact, r, dst)[...] = blk(C, r, dst) - prod
                mr, mi = mag(blk(C, r, src), T[p])
                check(blk(got, r, dst), blk(exact, r, dst), blk(C, r, dst), mr, mi, 128)
                touched[r, dst] = True
        for r in range(nb):
            for c in range(nb):
                if not touched[r, c]:
                    assert np.array_equal(blk(got, r, c), blk(C, r, c)), (mode, r, c)


def test_probe_rejects_bad_sizes(bg):
    with pytest.raises(bg.BEMError):
        bg.tc_probe(0, np.zeros((384, 384), complex), np.zeros((384, 128)), np.zeros((384, 128)))
    with pytest.raises(bg.BEMError):
        bg.tc_probe(9, np.zeros((512, 512), complex), np.zeros((512, 128)), np.zeros((512, 128)))
