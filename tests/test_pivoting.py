"""bem_dense_solve on matrices that need row exchanges.  The reference factorises
with Eigen::PartialPivLU (Solver_Base.h:85, Hydrodynamic_Solver.cpp:430); the
library's fast LU exchanges no rows and, when it meets a multiplier |l_ik| > 1 or a
zero pivot, factors the matrix again with partial pivoting (the first row of largest
|a_ij|, Eigen's rule).  Checked against numpy and the oracle's partial-pivot LU."""
import numpy as np
import pytest

from conftest import normwise

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


def _permuted(n, seed):
    """A diagonally dominant matrix with its rows shuffled: any LU without row
    exchanges meets tiny or zero pivots; with partial pivoting it is well conditioned."""
    rng = np.random.default_rng(seed)
    D = 0.5 * np.eye(n) + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    P = rng.permutation(n)
    B = rng.standard_normal((n, 4)) + 1j * rng.standard_normal((n, 4))
    return np.ascontiguousarray(D[P]), B


@pytest.mark.parametrize("n", [50, 300, 700])
def test_row_exchanges_plain_and_mixed(bg, orc, n):
    A, B = _permuted(n, n)
    ref = np.linalg.solve(A, B)
    assert normwise(orc.lu_solve(A, B), ref) < 1e-12
    for prec in (bg.PLAIN_FP64, bg.MIXED):
        x, it, res = bg.dense_solve(A, B, prec)
        print(n, prec, "iterations", it, "residual %.2e" % res, "err %.2e" % normwise(x, ref))
        assert normwise(x, ref) < 1e-11
        if prec == bg.PLAIN_FP64:
            assert it == 0 and res < 1e-13  # the direct pivoted solve
        else:
            # flexible GMRES behind the no-exchange TF32 factors may still converge (more
            # iterations); otherwise the pivoted fallback solves directly
            assert res <= 1e-12


def test_matrix_without_exchanges_keeps_the_fast_path(bg):
    rng = np.random.default_rng(5)
    n = 300
    A = 0.5 * np.eye(n) + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    B = rng.standard_normal((n, 3)) + 0j
    x, it, res = bg.dense_solve(A, B, bg.MIXED)
    assert it > 0 and res <= 1e-12  # refined TF32 factors, not the fallback
    assert normwise(x, np.linalg.solve(A, B)) < 1e-10


def test_singular_matrix_is_reported(bg):
    A, B = _permuted(64, 3)
    A[:, 17] = 0.0
    for prec in (bg.PLAIN_FP64, bg.MIXED):
        with pytest.raises(bg.BEMError) as ex:
            bg.dense_solve(A, B, prec)
        assert ex.value.status == 4 and "singular" in str(ex.value)
