"""Host mesh adaptation: fvmesh_adapt / fvmesh_transfer (meshadaptation.c,
criterionsmth.c, refineh_1.c, split.c, merge.c restated on the synthetic
host octree).

* a pass moves every leaf at most one level toward its target and keeps the
  2:1 face balance (fvmesh_flatten refuses an unbalanced mesh);
* split leaves hand their state to their children (split.c:493), so the
  volume integral of the state is unchanged;
* merged parents take the sum of their children's states each divided by 8
  in child order (merge.c:93-101), checked value for value;
* levels stay within [min_level, max_level]; the transfer refuses a state
  of the wrong size.
"""
import numpy as np
import pytest

from fv_140823_gb300.mesh import refine_by, uniform_mesh


def _integral(S, vol):
    return (S * vol).sum(axis=1)


def test_refinement_moves_one_level_and_injects_the_state():
    m = uniform_mesh(3, periodic=(1, 1, 1))
    t0 = m.flatten()
    rng = np.random.default_rng(0)
    S0 = rng.standard_normal((5, t0.ncells))
    level, cen = m.leaves()
    split = np.where(((cen - 0.5) ** 2).sum(axis=0) < 0.08, 6, 1).astype(np.int32)
    m.adapt(split, 3, 6)
    t1 = m.flatten()
    assert t1.level.max() == 4 and t1.level.min() == 3
    S1 = m.transfer(S0)
    # every new leaf carries the state of the old leaf that contains it
    pos0 = {(int(t0.ijk[0, i]), int(t0.ijk[1, i]), int(t0.ijk[2, i])): i for i in range(t0.ncells)}
    for i in range(t1.ncells):
        sh = t1.level[i] - 3
        key = tuple(int(t1.ijk[a, i]) >> sh for a in range(3))
        assert np.array_equal(S1[:, i], S0[:, pos0[key]])
    np.testing.assert_allclose(_integral(S1, t1.vol), _integral(S0, t0.vol), rtol=1e-13, atol=1e-13)


def test_merge_averages_the_children_in_child_order():
    m = uniform_mesh(2, periodic=(1, 1, 1))
    refine_by(m, lambda l, c: c[0] < 0.5, 3)
    t0 = m.flatten()
    assert t0.level.max() == 3
    rng = np.random.default_rng(1)
    S0 = rng.standard_normal((5, t0.ncells)) * 10.0 ** rng.integers(-3, 4, (5, t0.ncells))
    m.adapt(np.ones(t0.ncells, np.int32), 2, 5)
    t1 = m.flatten()
    assert t1.ncells == 64 and np.all(t1.level == 2)
    S1 = m.transfer(S0)
    pos0 = {(int(t0.level[i]), int(t0.ijk[0, i]), int(t0.ijk[1, i]), int(t0.ijk[2, i])): i
            for i in range(t0.ncells)}
    for i in range(t1.ncells):
        p = [int(t1.ijk[a, i]) for a in range(3)]
        if (2, *p) in pos0:  # unchanged leaf
            assert np.array_equal(S1[:, i], S0[:, pos0[(2, *p)]])
            continue
        want = np.zeros(5)
        for ch in range(8):
            k = pos0[(3, 2 * p[0] + (ch & 1), 2 * p[1] + ((ch >> 1) & 1), 2 * p[2] + ((ch >> 2) & 1))]
            want = want + S0[:, k] / 8.0
        assert np.array_equal(S1[:, i], want)
    np.testing.assert_allclose(_integral(S1, t1.vol), _integral(S0, t0.vol), rtol=1e-12)


@pytest.mark.parametrize("seed", [2, 3, 4])
def test_random_targets_keep_balance_and_bounds(seed):
    rng = np.random.default_rng(seed)
    m = uniform_mesh(3, side_bc=(2, 2, 2, 2, 2, 2))
    prev = None
    for _ in range(6):
        level, cen = m.leaves()
        n = level.size
        split = rng.integers(1, 8, n).astype(np.int32)
        m.adapt(split, 3, 6)
        t = m.flatten()   # raises when a face sees two levels
        assert t.level.min() >= 3 and t.level.max() <= 6
        S = m.transfer(np.tile(np.arange(n, dtype=np.float64), (5, 1)))
        assert S.shape == (5, t.ncells)
        if prev is not None:
            # one level per pass: a new leaf lies inside a former leaf at most
            # one level coarser, or is the parent of former leaves
            assert abs(int(t.level.max()) - int(prev)) <= 1
        prev = t.level.max()


def test_transfer_rejects_a_state_of_the_wrong_size():
    m = uniform_mesh(2)
    n = m.ncells
    m.adapt(np.full(n, 3, np.int32), 2, 3)
    with pytest.raises(RuntimeError):
        m.transfer(np.zeros((5, n + 1)))
    with pytest.raises(RuntimeError):
        m.adapt(np.zeros(m.ncells, np.int32), 4, 3)
