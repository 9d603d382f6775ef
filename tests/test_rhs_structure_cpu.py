"""Properties of the reference's transient right-hand side that the chained step start relies on,
checked on the oracle (CPU): the non-Dirichlet rows of b are linear in the previous solution and
read it on non-Dirichlet rows only, and the Dirichlet rows depend on the field alone.  So with
the field unchanged b - b' = S (x_n - x_(n-1)), S the field-free map (the step start forms it in
double-float from the edge sigma), and the node right-hand-side kernel may write the Dirichlet
values into the vector it reads x_prev from."""
import numpy as np
import pytest

import qms_oracle as o

CASES = [(10, 9, 11, 1e-5, 3), (7, 12, 8, 2.7e-5, 8)]
V, B, G = (1.5, -0.5, 0.25), (2e-3, -1e-3, 5e-3), [0.05, 0.02, -0.01, 0.02, -0.03, 0.04, -0.01, 0.04, -0.02]


def setup(xs, ys, zs, seed):
    rng = np.random.default_rng(seed)
    geom = rng.integers(0, 4, size=(xs, ys, zs)).astype(np.float64).flatten(order="F")
    props = np.array([[m + 1, *(10 ** rng.uniform(0, 3, 3)), *(10 ** rng.uniform(5, 7.7, 3))] for m in range(3)])
    return o.materials(xs, ys, zs, geom, props), rng


def dirichlet_mask(ia, ja, a):
    """Rows that are identity rows of the assembled matrix (the Dirichlet shell)."""
    n = ia.size - 1
    first = ia[:-1] - 1
    single = np.diff(ia) == 1
    mask = np.zeros(n, bool)
    r = np.nonzero(single)[0]
    mask[r] = (ja[first[r]] - 1 == r) & (a[first[r]] == 1.0)
    return mask


@pytest.mark.parametrize("xs,ys,zs,dt,seed", CASES)
def test_rhs_change_is_the_field_free_map_of_the_state_change(xs, ys, zs, dt, seed):
    c, rng = setup(xs, ys, zs, seed)
    d = (1e-3, 1.1e-3, 0.9e-3)
    n = o.sizes(xs, ys, zs)[0]
    x1, x2 = rng.standard_normal(n) * 1e-3, rng.standard_normal(n) * 1e-3
    ia, ja, a, b1 = o.assemble(xs, ys, zs, *d, c, True, dt, V, B, G, x_prev=x1)
    _, _, _, b2 = o.assemble(xs, ys, zs, *d, c, True, dt, V, B, G, x_prev=x2)
    _, _, _, s = o.assemble(xs, ys, zs, *d, c, True, dt, V, np.zeros(3), np.zeros(9), x_prev=x1 - x2)
    fixed = dirichlet_mask(ia, ja, a)
    assert fixed.any() and not fixed.all()
    assert np.array_equal(b1[fixed], b2[fixed])           # the lift: the field alone
    assert not s[fixed].any()
    scale = np.abs(b1).max()
    assert np.abs((b1 - b2) - s)[~fixed].max() <= 1e-12 * scale


@pytest.mark.parametrize("xs,ys,zs,dt,seed", CASES)
def test_rhs_reads_the_state_on_non_dirichlet_rows_only(xs, ys, zs, dt, seed):
    c, rng = setup(xs, ys, zs, seed)
    d = (1e-3, 1.1e-3, 0.9e-3)
    n = o.sizes(xs, ys, zs)[0]
    x = rng.standard_normal(n) * 1e-3
    ia, ja, a, b = o.assemble(xs, ys, zs, *d, c, True, dt, V, B, G, x_prev=x)
    fixed = dirichlet_mask(ia, ja, a)
    y = x.copy()
    y[fixed] += rng.standard_normal(int(fixed.sum()))      # change the state on the Dirichlet rows only
    _, _, _, b_y = o.assemble(xs, ys, zs, *d, c, True, dt, V, B, G, x_prev=y)
    assert np.array_equal(b, b_y)
