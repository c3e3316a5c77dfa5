"""A planar-target view for the differentiable-path tests (CPU side).

Renders a seeded pose of the planar target on the config-1 rig at a reduced
size, decodes it with the FP64 oracle, and prepares everything the oracle's
differentiable forward needs: its own rectification (fixed geometry), the
nominal parameters, match columns from its own rectify + stereoMatch, and the
target plane in the rectified left frame.
"""
import math

import numpy as np

from oracle import oracle as O
from zim_gb300 import synth

TWO_PI = 2 * math.pi


class DiffCase:
    def __init__(self, width=320, height=256, pose=0, seed=3):
        spec = synth.pose_plane(seed=seed, width=width, height=height, pose=pose)
        self.spec = spec
        self.L = spec.render(0)
        self.R = spec.render(1)
        cfg = O.make_decode_cfg(**spec.decode_kwargs())
        self.order, self.residual = [], []
        for frames in (self.L, self.R):
            ph, k, _, valid, _ = O.decode(cfg, frames)
            res = np.where(valid > 0, ph - TWO_PI * k, 0.0)
            self.order.append(np.where(valid > 0, k, 0).astype(np.int32))
            self.residual.append(res)
        rig = spec.rig
        calib = O.make_calib(rig.K, rig.D, rig.R, rig.t, rig.width, rig.height)
        R1, R2, P1, P2, Q, rw, rh = O.rectification(calib)
        self.R1, self.Q, self.rect_w, self.rect_h = R1, Q, rw, rh
        ir = [np.linalg.inv(P1[:, :3] @ R1), np.linalg.inv(P2[:, :3] @ R2)]
        dist = [(rig.D[c][2], rig.D[c][3], rig.D[c][4]) for c in range(2)]
        self.baseline0 = float(np.linalg.norm(rig.t))
        self.geom = O.diff_geom(ir, dist, Q, self.baseline0, rw, rh, rig.width, rig.height)
        self.theta0 = np.array([v for c in range(2) for v in (rig.K[c][0, 0], rig.K[c][1, 1], rig.K[c][0, 2],
                                                              rig.K[c][1, 2], rig.D[c][0], rig.D[c][1])]
                               + [self.baseline0, 0.0, 0.0, 0.0])
        # match columns from the oracle's standard setData + stereoMatch
        ph = []
        for c, (P, Rc) in enumerate(((P1, R1), (P2, R2))):
            mx, my = O.init_rectify_map(rig.K[c], rig.D[c], Rc, P, rw, rh)
            full = TWO_PI * self.order[c] + self.residual[c]
            ph.append((O.remap_linear(full, mx, my), O.remap_nearest(self.order[c], mx, my)))
        _, self.best, _ = O.stereo_match(ph[0][0], ph[1][0], ph[0][1], ph[1][1], spec.pha_f)
        n = np.asarray(spec.plane_n, np.float64)
        self.plane = np.concatenate([R1 @ n, [-spec.plane_d]])

    def eval(self, theta, **kw):
        return O.diff_eval(self.geom, theta, self.order[0], self.residual[0], self.order[1], self.residual[1],
                           self.best, self.plane, **kw)


def fd_step(theta):
    """Central-difference steps: 1e-4 relative, or absolute for parameters at 0
    (or small distortion terms)."""
    h = 1e-4 * np.abs(theta)
    h[4], h[5], h[10], h[11] = 1e-6, 1e-6, 1e-6, 1e-6  # k1, k2 of both cameras
    h[13:] = 1e-6                                     # rotation update (rad)
    return h
