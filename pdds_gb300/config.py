"""Workload definitions and the RBF shape rule.

The reference sets the Gaussian RBF shape c of a stencil side from fac[kind]
(Meshes/stencil.cpp:211-243); its configuration.txt uses
fac = 1.5 1.27 1.2 1.13 at a knot spacing of 10/28, i.e. c = kappa * spacing
with kappa = (4.2, 3.556, 3.36, 3.164) for side kinds 0..3 (one interface with
one elongation ... two interfaces with two elongations).  fac_rule keeps those
ratios for any layout, which keeps cond(Psi) near the reference's 1e9..1e11.
"""
from __future__ import annotations

REF_FAC = (1.5, 1.27, 1.2, 1.13)
REF_SPACING = 10.0 / 28.0
KAPPA = tuple(f / REF_SPACING for f in REF_FAC)


def fac_rule(side_length: float, nsub: int, nnode: int):
    """fac[kind] = kappa[kind] * knot spacing for a square layout of side length L.

    With more than 16 knots per segment the sides hold 45..130 knots and the
    kind 0..2 ratios push cond(Psi) past 1e12 (4e13 for the 84-knot sides of
    43-knot segments, where two inverse algorithms then disagree by 1e-4 in
    the cardinal weights); there every kind uses the kind-3 ratio 3.164,
    which keeps cond(Psi) near 4e10."""
    gap = side_length / ((nnode - 1) * nsub)
    kappa = KAPPA if nnode <= 16 else (KAPPA[3],) * 4
    return tuple(k * gap for k in kappa)


# The synthetic workloads of the benchmark configurations.
WORKLOADS = {
    # 2-D Poisson on [-1,1]^2, u = sin(pi x)cos(pi y) + xy, 4x4 subdomains, 11 knots per segment
    "poisson_4x4_n11": dict(sw=(-1.0, -1.0), ne=(1.0, 1.0), nsub=4, nnode=11, npaths=10_000, h=1e-3),
    # the same problem scaled up: 12x12 subdomains, 43 knots per segment
    "poisson_12x12_n43": dict(sw=(-1.0, -1.0), ne=(1.0, 1.0), nsub=12, nnode=43, npaths=20_000, h=5e-4),
    # variable coefficients on [0,1]^2 served from 1024^2 FP32 tables, 8x8 subdomains, 31 knots per segment
    "varcoef_lut_8x8_n31": dict(sw=(0.0, 0.0), ne=(1.0, 1.0), nsub=8, nnode=31, npaths=50_000, h=5e-4,
                                problem="varcoef_lut", lut_n=1024),
}


def varcoef_tables(n: int = 1024, bounds=(0.0, 0.0, 1.0, 1.0)):
    """Coefficient and boundary tables of the variable-coefficient problem
    0.5 sum (sigma sigma^T)_ij d_ij u + b.grad u + c u + f = 0 with
    sigma = diag(1 + x^2/2, 1 + y^2/2), b = (y, -x), c = -(1 + x^2 + y^2),
    u = exp(x) cos(2y) + 1 and f derived from u, sampled on an n x n grid
    over bounds (x0, y0, x1, y1) in FP32.  Fields per node: sigma11, sigma22,
    b1, b2, c, f, du/dx, du/dy.  Returns (coef [n][n][8], g [n][n], bounds)."""
    import numpy as np
    x0, y0, x1, y1 = bounds
    xs = x0 + (x1 - x0) * np.arange(n) / (n - 1)
    ys = y0 + (y1 - y0) * np.arange(n) / (n - 1)
    X, Y = np.meshgrid(xs, ys)  # [ny][nx]
    s1 = 1.0 + 0.5 * X * X
    s2 = 1.0 + 0.5 * Y * Y
    ex = np.exp(X)
    ux = ex * np.cos(2 * Y)
    uy = -2.0 * ex * np.sin(2 * Y)
    uxx, uyy = ux, -4.0 * ux
    c = -(1.0 + X * X + Y * Y)
    u = ux + 1.0
    f = -(0.5 * (s1 * s1 * uxx + s2 * s2 * uyy) + (Y * ux - X * uy) + c * u)
    coef = np.stack([s1, s2, Y, -X, c, f, ux, uy], axis=-1).astype(np.float32)
    return np.ascontiguousarray(coef), np.ascontiguousarray(u.astype(np.float32)), tuple(float(b) for b in bounds)


def layout_knot_count(nsub: int, nnode: int) -> int:
    """Knots of an nsub x nsub layout with nnode knots per interface segment
    (shared cross knots counted once): (g-1)(g(n-1)+1) + (g-1)(g(n-2)+2)."""
    g, n = int(nsub), int(nnode)
    return (g - 1) * (g * (n - 1) + 1) + (g - 1) * (g * (n - 2) + 2)


def instance_step(g: int, h_ref: float = 1e-3, g_ref: int = 4) -> float:
    """Step of an instance with g x g subdomains on the unit square: h_ref at
    g_ref x g_ref, scaled with the square of the subdomain size above it, so
    sqrt(h) stays the same fraction of a subdomain (the step's bias is a
    function of that ratio) and paths take the same number of steps."""
    return h_ref * min(1.0, (g_ref / g) ** 2)


def batch_instances(n: int = 256, seed: int = 1234, grid=(4, 16), nodes=(11, 41), scaled_h: float = 0.0):
    """The many-instance workload: n Helmholtz problems Lap u + c u + f = 0
    on [0,1]^2 with u = sin(a x) cos(b y), a, b ~ U[1,4], c ~ U[-4,0], each
    on its own g x g subdomain grid, g ~ U{4..16}, with k ~ U{11..41} knots
    per segment (seeded).  The grids are square: the reference's layout
    (Fullfill_interfaces and its configuration reader) takes one subdomain
    count for both directions.  scaled_h > 0 gives each instance the step
    instance_step(g, scaled_h) (0: the run's step for all)."""
    import numpy as np
    from .api import Instance
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        g = int(rng.integers(grid[0], grid[1] + 1))
        k = int(rng.integers(nodes[0], nodes[1] + 1))
        a, b = rng.uniform(1.0, 4.0, size=2)
        c = -rng.uniform(0.0, 4.0)
        out.append(Instance((0.0, 0.0), (1.0, 1.0), g, k, fac_rule(1.0, g, k), (float(a), float(b), float(c)),
                            instance_step(g, scaled_h) if scaled_h > 0 else 0.0))
    return out
