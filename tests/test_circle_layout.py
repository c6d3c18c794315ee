"""Circle layout (disk split into rings x sectors) on the host: knot count
and placement, boundary knots, every knot inside its polar stencil, side
knots on their arcs and rays, G rows = the union of the stencil's side
knots, and the RBF side matrices well conditioned."""
import numpy as np
import pytest

import pdds_gb300 as P

NR, NS, N = 6, 16, 11


@pytest.fixture(scope="module")
def pd():
    from pdds_gb300 import build as B
    B.build()
    d = P.PDDSparseGM.circle_mesh(1.0, NR, NS, N, device=-1)
    yield d
    d.close()


def polar_outside(rect, x, y):
    r0, p0, r1, p1 = rect
    rho = np.hypot(x, y)
    d = [rho - r1]
    if p1 - p0 < 6.2:
        d += [np.sin(p0) * x - np.cos(p0) * y, np.cos(p1) * y - np.sin(p1) * x]
    if r0 > 0:
        d.append(r0 - rho)
    return max(d)


def test_knots(pd):
    K = (NR - 1) * NS * (N - 1) + (NR - 1) * NS * (N - 2) + NS  # no rays in the central disk
    assert pd.K == K
    r = np.hypot(pd.x, pd.y)
    assert r.max() <= 1.0 + 1e-12 and r.min() > 0.0
    assert pd.layout_info["nboundary"] == NS
    assert np.sum(np.abs(r - 1.0) < 1e-12) == NS
    # rings: every knot lies on an arc between rings or on a ray between sectors
    on_arc = np.abs(r * NR - np.round(r * NR)) < 1e-9
    ang = np.mod(np.arctan2(pd.y, pd.x), 2 * np.pi) * NS / (2 * np.pi)
    on_ray = np.abs(ang - np.round(ang)) < 1e-9
    assert np.all(on_arc | on_ray)


def test_stencils_and_rows(pd):
    inner = np.abs(np.hypot(pd.x, pd.y) - 1.0) > 1e-12
    for k in np.where(inner)[0]:
        rect, kinds, sides = pd.stencil(int(k))
        assert polar_outside(rect, pd.x[k], pd.y[k]) < -1e-6, k
        r0, p0, r1, p1 = rect
        cols = set()
        for d, idx in enumerate(sides):
            if len(idx) == 0:
                continue
            cols.update(idx.tolist())
            xs, ys = pd.x[idx], pd.y[idx]
            if d <= 1:  # arcs: N at rho1, S at rho0
                assert np.allclose(np.hypot(xs, ys), r1 if d == 0 else r0, atol=1e-12)
            else:       # rays: E at phi1, W at phi0
                phi = p1 if d == 2 else p0
                assert np.allclose(np.cos(phi) * ys - np.sin(phi) * xs, 0.0, atol=1e-12)
            assert 0 <= kinds[d] <= 3
        a, b = pd.row_ptr[k], pd.row_ptr[k + 1]
        assert sorted(cols) == pd.col[a:b].tolist()
        assert (r0 == 0.0) == (len(sides[1]) == 0)     # no inner arc at the centre
        if p1 - p0 > 6.2:  # the central disk's stencil: one periodic arc, no rays
            assert len(sides[2]) == 0 and len(sides[3]) == 0 and len(sides[0]) == NS * (N - 1)
        assert (abs(r1 - 1.0) < 1e-12) == (len(sides[0]) == 0)  # outer arc on the boundary: no knots


def test_side_matrices_conditioned(pd):
    seen = 0
    for k in range(0, pd.K, 37):
        if abs(np.hypot(pd.x[k], pd.y[k]) - 1.0) < 1e-12:
            continue
        rect, kinds, sides = pd.stencil(int(k))
        for d, idx in enumerate(sides):
            if len(idx) < 2:
                continue
            p = np.stack([pd.x[idx], pd.y[idx]], 1)
            gap = np.min(np.linalg.norm(np.diff(p, axis=0), axis=1))
            c = 3.164 * gap
            D2 = ((p[:, None, :] - p[None, :, :]) ** 2).sum(-1)
            cond = np.linalg.cond(np.exp(-D2 / c ** 2))
            assert cond < 1e12, (k, d, cond)
            seen += 1
    assert seen > 20
