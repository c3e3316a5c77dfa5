"""Coefficient maps for the per-pixel polynomial reprojection
(evaluateV2CalibPoint, JSLAB_PhaseEpipolarReconstructor_V2.cpp:13-76).

``random_maps`` mixes every model branch the reference evaluates, plus the
rejections (all-zero z map, vanishing denominators, non-finite values), for bit-exact
parity.  ``q_maps`` builds maps of one model that reproduce the Q-matrix
reprojection of a rectified rig up to float rounding of the coefficients.
"""
import numpy as np

INV, RAY, LIN, RAT = -1.0, -2.0, -3.0, -4.0
BRANCHES = ("inv_cubic", "ray_inv", "ray_cubic", "lin_rational", "lin_cubic", "z_inv", "cubic", "zero",
            "inv_zero_den", "rat_zero_den", "inv_inf", "nonfinite")
UNIT_D = ("inv_zero_den", "rat_zero_den")  # pixels whose disparity is set to 1


def random_maps(h, w, seed=0, d_scale=100.0):
    """(cx, cy, cz) float32 (h, w, 4) and the branch index per pixel.  Scaled
    so disparities near d_scale give depths of a few hundred units."""
    rng = np.random.default_rng(seed)
    br = rng.integers(0, len(BRANCHES), size=(h, w))
    cx = rng.normal(0, 1, (h, w, 4)).astype(np.float32)
    cy = rng.normal(0, 1, (h, w, 4)).astype(np.float32)
    cz = rng.normal(0, 1, (h, w, 4)).astype(np.float32)
    s = 1.0 / d_scale
    # keep the untagged c3 away from the tags
    cx[..., 3] = np.where(np.abs(cx[..., 3]) > 0.5, 0.3, cx[..., 3]).astype(np.float32)
    cz[..., 3] = np.where(np.abs(cz[..., 3]) > 0.5, 0.3, cz[..., 3]).astype(np.float32)

    def put(name, x=None, y=None, z=None):
        m = br == BRANCHES.index(name)
        for arr, v in ((cx, x), (cy, y), (cz, z)):
            if v is not None:
                for c, val in enumerate(v):
                    if val is not None:
                        arr[..., c][m] = val if np.isscalar(val) else val[m]
    u = lambda lo, hi: rng.uniform(lo, hi, (h, w)).astype(np.float32)
    # inverse depth 1/z = a + b d (+ tiny cubic terms)
    put("inv_cubic", x=(u(-1, 1), None, None, INV), z=(u(1e-4, 1e-3), u(1e-5, 3e-5), u(-1e-9, 1e-9), u(-1e-12, 1e-12)))
    put("ray_inv", x=(u(-1, 1), None, None, RAY), z=(u(1e-4, 1e-3), u(1e-5, 3e-5), u(-1e-9, 1e-9), INV))
    put("ray_cubic", x=(u(-1, 1), None, None, RAY), z=(u(100, 900), u(-2, 2), u(-1e-3, 1e-3), u(-1e-6, 1e-6)))
    put("lin_rational", x=(u(-1, 1), u(-5, 5), None, LIN), y=(u(-1, 1), u(-5, 5), None, None),
        z=(u(500, 2000), u(s, 3 * s), None, RAT))
    put("lin_cubic", x=(u(-1, 1), u(-5, 5), None, LIN), z=(u(100, 900), u(-2, 2), u(-1e-3, 1e-3), u(-1e-6, 1e-6)))
    put("z_inv", x=(None, None, None, 0.25), z=(u(1e-4, 1e-3), u(1e-5, 3e-5), u(-1e-9, 1e-9), INV))
    put("cubic", x=(u(-500, 500), u(-1, 1), u(-1e-3, 1e-3), u(-1e-6, 1e-6)),
        y=(u(-500, 500), u(-1, 1), u(-1e-3, 1e-3), u(-1e-6, 1e-6)),
        z=(u(100, 900), u(-2, 2), u(-1e-3, 1e-3), u(-1e-6, 1e-6)))
    put("zero", z=(0.0, 0.0, 5e-10, -5e-10))
    # 1/z = 1 - d and den = 1 - d vanish at d = 1 (random_disparity puts d = 1 there)
    put("inv_zero_den", x=(None, None, None, INV), z=(1.0, -1.0, 0.0, 0.0))
    put("rat_zero_den", x=(None, None, None, LIN), z=(1.0, -1.0, 0.0, RAT))
    put("inv_inf", x=(None, None, None, INV), z=(1.0, np.inf, 0.0, 0.0))
    put("nonfinite", x=(np.nan, None, None, 0.125), z=(500.0, 0.0, 0.0, 0.0))
    return cx, cy, cz, br


def random_disparity(h, w, br=None, seed=1, d_scale=100.0):
    rng = np.random.default_rng(seed)
    d = rng.uniform(0.5 * d_scale, 1.5 * d_scale, (h, w)).astype(np.float32)
    d[rng.random((h, w)) < 0.1] = 0.0
    d[rng.random((h, w)) < 0.02] = np.float32(1e-5)  # at the |d| < 1e-5 gate
    d[rng.random((h, w)) < 0.02] = -d_scale
    if br is not None:
        for name in UNIT_D:
            d[br == BRANCHES.index(name)] = 1.0
    return d


def q_maps(Q, h, w, model="inv"):
    """Maps reproducing x=(j+Q03)/wq, y=(i+Q13)/wq, z=Q23/wq with wq = Q32 d + Q33.
    model: "inv" (x-tag -1), "ray" (x-tag -2, z-tag -1), "zinv" (z-tag -1),
    "rational" (x-tag -3, z-tag -4; needs Q33 != 0)."""
    Q = np.asarray(Q, np.float64).reshape(4, 4)
    j = np.arange(w, dtype=np.float64)[None, :].repeat(h, 0)
    i = np.arange(h, dtype=np.float64)[:, None].repeat(w, 1)
    cx = np.zeros((h, w, 4), np.float64)
    cy = np.zeros((h, w, 4), np.float64)
    cz = np.zeros((h, w, 4), np.float64)
    cx[..., 0] = (j + Q[0, 3]) / Q[2, 3]
    cy[..., 0] = (i + Q[1, 3]) / Q[2, 3]
    if model == "rational":
        cz[..., 0] = Q[2, 3] / Q[3, 3]
        cz[..., 1] = Q[3, 2] / Q[3, 3]
        cx[..., 3], cz[..., 3] = LIN, RAT
    else:
        cz[..., 0] = Q[3, 3] / Q[2, 3]
        cz[..., 1] = Q[3, 2] / Q[2, 3]
        if model == "inv":
            cx[..., 3] = INV
        elif model == "ray":
            cx[..., 3], cz[..., 3] = RAY, INV
        elif model == "zinv":
            cz[..., 3] = INV
        else:
            raise ValueError(model)
    return cx.astype(np.float32), cy.astype(np.float32), cz.astype(np.float32)
