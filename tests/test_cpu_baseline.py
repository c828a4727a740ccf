"""The CPU baseline's sampled product (test infrastructure of the reference arm):
the layered, BLAS-backed leaf products of oracle/oracle.c (mltaGeM_ per leaf,
H/mblock.cpp:141-154, 225-238; threads share row-disjoint groups) equal the
oracle's plain product, with and without the host BLAS, for one and several
right-hand sides, on the whole leaf set and on a sample of it."""
import numpy as np
import pytest

import oracle as O


@pytest.fixture(scope="module")
def fib(golden):
    g = golden("fib4096")
    Ho = O.OracleH(g["points"], O.TREE_BBX, 32, 0.8, float(g["h"]))
    Ho.assemble(1e-6, nthreads=4)
    return Ho


@pytest.mark.parametrize("blas", [False, True])
@pytest.mark.parametrize("p", [1, 16])
def test_layered_product_equals_plain_product(fib, blas, p):
    Ho = fib
    if blas and O.use_host_blas() is None:
        pytest.skip("no host BLAS")
    if not blas:
        O.lib().or_set_blas(None, None)
    X = np.random.default_rng(p).uniform(-1, 1, (p, Ho.n))
    X = X[0].copy() if p == 1 else X
    Yo = Ho.matvec(X, np.zeros_like(X), d=0.5)
    plan = O.layered_groups(Ho.leaves(), np.arange(Ho.nleaves))
    Y = Ho.matvec_layers(plan, X, np.zeros_like(X), d=0.5, nthreads=4)
    assert np.linalg.norm(Y - Yo) / np.linalg.norm(Yo) < 1e-13
    O.lib().or_set_blas(None, None)


def test_layers_are_row_disjoint_and_cover_the_sample(fib):
    lv = fib.leaves()
    sel = np.random.default_rng(0).choice(len(lv), len(lv) // 8, replace=False)
    order, gs, ls = O.layered_groups(lv, sel)
    assert sorted(order.tolist()) == sorted(sel.tolist())
    for q in range(len(ls) - 1):
        spans = sorted((int(lv[order[gs[g]], 0]), int(lv[order[gs[g]], 0] + lv[order[gs[g]], 1]))
                       for g in range(ls[q], ls[q + 1]))
        for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
            assert a1 <= b0
