"""Invariants of the flattened octree tables (host mesh builder)."""
import numpy as np
import pytest

from fv_140823_gb300.mesh import FACE_AXIS, FACE_OPP, FACE_SIGN, HANG0, refine_by, uniform_mesh


def amr(periodic=(0, 0, 0), base=2, maxl=5, seed=0):
    rng = np.random.default_rng(seed)
    c0 = rng.uniform(0.2, 0.8, 3)
    m = uniform_mesh(base, periodic=periodic)
    refine_by(m, lambda l, c: ((c - c0[:, None]) ** 2).sum(0) < 0.02 * (maxl - l + 1), maxl)
    return m


@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 1, 1), (0, 1, 0)])
def test_links_reciprocal_and_balanced(periodic):
    t = amr(periodic).flatten()
    n = t.ncells
    for f in range(6):
        for c in range(n):
            code = t.nbr[f, c]
            if -8 <= code < 0:
                axis = FACE_AXIS[f]
                assert not periodic[axis]
                continue
            nf = t.nbr_face[f, c]
            assert nf == FACE_OPP[f]
            if code >= 0:
                assert abs(int(t.level[code]) - int(t.level[c])) <= 1
                back = t.nbr[nf, code]
                if back >= 0:
                    assert back == c
                else:
                    assert back <= HANG0 and c in t.hang_nbr[HANG0 - back]
            else:
                r = HANG0 - code
                assert t.hang_cell[r] == c and t.hang_face[r] == f
                for k in t.hang_nbr[r]:
                    assert t.level[k] == t.level[c] + 1
                    assert t.nbr[nf, k] == c


# fcnd2elnd (operatetp.c:113-147, type 0): element node of face f at face
# node s; node n sits at offset (n & 1, n >> 1 & 1, n >> 2 & 1) in (x, y, z).
FACE_NODES = [[0, 1, 5, 4], [3, 7, 5, 1], [2, 6, 7, 3], [2, 0, 4, 6], [2, 3, 1, 0], [6, 4, 5, 7]]


@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 1, 1)])
def test_hanging_neighbours_in_face_node_order(periodic):
    """Fine neighbour s of a 1:4 face holds the coarse face's node s as a corner
    (the order elconnfin.c:42-45 gives neigtr[f][s], and so the order in which
    the four sub-face fluxes are summed)."""
    t = amr(periodic).flatten()
    nl = {int(l): 1 << int(l) for l in np.unique(t.level)}
    for r in range(t.nhang):
        c, f = int(t.hang_cell[r]), int(t.hang_face[r])
        l = int(t.level[c])
        for s in range(4):
            node = FACE_NODES[f][s]
            corner = [2 * (int(t.ijk[x, c]) + ((node >> x) & 1)) for x in range(3)]  # fine lattice
            k = int(t.hang_nbr[r, s])
            lo = [int(t.ijk[x, k]) for x in range(3)]
            d = [corner[x] - lo[x] for x in range(3)]
            # the corner lies on the fine cell's closed extent, modulo a periodic wrap
            d = [d[x] % (2 * nl[l]) if periodic[x] else d[x] for x in range(3)]
            assert all(v in (0, 1) for v in d), (r, s, c, f, k)
        assert len(set(int(k) for k in t.hang_nbr[r])) == 4


def test_volumes_and_areas():
    m = amr((1, 0, 1))
    t = m.flatten()
    assert t.vol.sum() == pytest.approx(1.0, rel=0, abs=1e-14)
    h = np.ldexp(1.0, -t.level.astype(np.int64))
    # six tetrahedra as meshproperties.c:66-111 sums them: within an ulp or two of h^3
    np.testing.assert_allclose(t.vol, h * h * h, rtol=5e-16, atol=0)
    for r in range(t.nhang):
        c, f = t.hang_cell[r], t.hang_face[r]
        assert t.hang_area[r].sum() == t.area[f, c]


def test_morton_order_and_levels():
    t = amr().flatten()
    shift = 18 - t.level.astype(np.int64)

    def spread(x):
        out = np.zeros_like(x)
        for b in range(21):
            out |= ((x >> b) & 1) << (3 * b)
        return out

    key = spread(t.ijk[0].astype(np.int64) << shift) | (spread(t.ijk[1].astype(np.int64) << shift) << 1) | (
        spread(t.ijk[2].astype(np.int64) << shift) << 2)
    assert np.all(np.diff(key) > 0)


def test_leaf_cells_equal_the_flattened_leaf_list():
    m = amr()
    level, ijk = m.leaf_cells()
    t = m.flatten()
    assert np.array_equal(level, t.level) and np.array_equal(ijk, t.ijk)


def test_uniform_distances_follow_distance_c():
    # distance.c, same level: dist_cc = |dx| / 2, dist_cf = |dx| / 4
    t = uniform_mesh(4, periodic=(1, 1, 1)).flatten()
    h = 1.0 / 16
    assert np.all(t.dcc == 0.5 * h) and np.all(t.dcf == 0.25 * h)
    assert np.all(t.nbr >= 0)


def test_boundary_faces_have_zero_distance():
    t = uniform_mesh(3).flatten()
    b = (t.nbr < 0) & (t.nbr > HANG0)
    assert b.sum() == 6 * 64
    assert np.all(t.dcc[b] == 0) and np.all(t.dcf[b] == 0)
    assert np.all(t.nbr[b] == -3)  # transmissive, bc code 2


def test_refinement_balance_enforced_across_periodic_wrap():
    m = uniform_mesh(2, periodic=(1, 1, 1))
    refine_by(m, lambda l, c: (c[0] < 0.1) & (c[1] < 0.1) & (c[2] < 0.1), 6)
    t = m.flatten()
    for f in range(6):
        code = t.nbr[f]
        ok = code >= 0
        assert np.all(np.abs(t.level[code[ok]] - t.level[ok]) <= 1)


def test_face_frames_orthonormal_and_outward():
    t = uniform_mesh(2).flatten()
    for f in range(6):
        n, t1, t2 = t.frames[f, :3], t.frames[f, 3:6], t.frames[f, 6:]
        assert n[FACE_AXIS[f]] == FACE_SIGN[f]
        assert np.dot(n, t1) == 0 and np.dot(n, t2) == 0 and np.dot(t1, t2) == 0
        assert np.array_equal(np.cross(n, t1), t2)
