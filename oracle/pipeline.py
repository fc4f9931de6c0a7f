"""CPU oracle of the whole per-frame loop (TEST INFRASTRUCTURE ONLY).

Same stage order and parameters as include/tde_pipeline.h, built from the
oracle's C stages: bilateral filter, pyramid, vertex maps, FP64 PCA normals,
coarse-to-fine ICP with FP64 sums and FP64 Cholesky / SO(3) update,
integration of the raw depth, raycast and model-map pyramid.
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc


class OraclePipeline:
    def __init__(self, cfg, pose12, levels=3):
        self.cfg = cfg
        self.levels = levels
        self.intr = orc.Intr(cfg.fx, cfg.fy, cfg.cx, cfg.cy, cfg.cols, cfg.rows)
        self.rb = orc.make_rb((cfg.voxels,) * 3, (cfg.volume_m,) * 3)
        self.vol = np.zeros(orc.volume_bytes(cfg.tsdf_format, self.rb), np.uint8)
        self.cell = np.full(3, cfg.cell, np.float32)
        self.R = np.asarray(pose12[:9], np.float64).reshape(3, 3).copy()
        self.t = np.asarray(pose12[9:12], np.float64).copy()
        self.frames = 0
        self.vmod = [None] * levels
        self.nmod = [None] * levels
        self.lost = []

    def frame_maps(self, depth):
        c = self.cfg
        d = orc.bilateral(depth, c.sigma_space, c.sigma_color, c.max_depth_mm)
        ds, vs, ns = [d], [], []
        for l in range(1, self.levels):
            ds.append(orc.pyramid(ds[-1], c.sigma_color))
        for l in range(self.levels):
            v = orc.vertex_map(ds[l], self.intr.level(l))
            vs.append(v)
            ns.append(orc.normal_map(v))
        return ds, vs, ns

    def track(self, vs, ns):
        c = self.cfg
        R_prev, t_prev = self.R.copy(), self.t.copy()
        R, t = self.R.copy(), self.t.copy()
        ok = True
        for l in range(self.levels - 1, -1, -1):
            il = self.intr.level(l)
            for _ in range(c.icp_iters[l]):
                pose24 = np.concatenate([R.astype(np.float32).ravel(), t.astype(np.float32),
                                         R_prev.T.astype(np.float32).ravel(), t_prev.astype(np.float32)])
                sums, _ = orc.icp_terms(vs[l], ns[l], self.vmod[l], self.nmod[l], pose24, il, c.dist_thresh,
                                        c.angle_thresh)
                if sums[27] < 6:
                    ok = False
                    continue
                st, R2, t2, _ = orc.icp_solve(sums, R.ravel(), t)
                if st != 0:
                    ok = False
                    continue
                R, t = R2.reshape(3, 3), t2
        if ok:
            self.R, self.t = R, t
        return ok

    def process(self, depth):
        c = self.cfg
        ds, vs, ns = self.frame_maps(depth)
        ok = True
        if self.frames > 0:
            ok = self.track(vs, ns)
        self.lost.append(not ok)
        Rf = self.R.astype(np.float32)
        tf = self.t.astype(np.float32)
        sd = orc.scale_depth(depth, self.intr)
        orc.integrate(sd, self.vol, c.tsdf_format, c.trunc_m, np.ascontiguousarray(Rf.T), tf, self.intr, self.cell,
                      self.rb, c.max_weight)
        vm, nm = orc.raycast(self.vol, c.tsdf_format, self.rb, self.intr, Rf, tf, c.trunc_m, self.cell)
        self.vmod[0], self.nmod[0] = vm, nm
        for l in range(1, self.levels):
            self.vmod[l] = orc.resize_map(self.vmod[l - 1], False)
            self.nmod[l] = orc.resize_map(self.nmod[l - 1], True)
        self.frames += 1
        return np.concatenate([self.R.ravel(), self.t])


class OraclePipelineF64(OraclePipeline):
    """The same loop with a full-FP64 model: FP64 TSDF values (int32 weights,
    no storage rounding), FP64 integration and raycast, FP64 ICP terms, sums
    and solve.  The reference point of the storage precision study."""

    def __init__(self, cfg, pose12, levels=3):
        super().__init__(cfg, pose12, levels)
        n = cfg.voxels ** 3
        self.vol = None
        self.tsdf = np.zeros(n, np.float64)
        self.weight = np.zeros(n, np.int32)
        self.cell64 = np.full(3, cfg.volume_m / cfg.voxels, np.float64)

    def track(self, vs, ns):
        c = self.cfg
        R_prev, t_prev = self.R.copy(), self.t.copy()
        R, t = self.R.copy(), self.t.copy()
        ok = True
        for l in range(self.levels - 1, -1, -1):
            il = self.intr.level(l)
            for _ in range(c.icp_iters[l]):
                sums = orc.icp_terms_f64(vs[l], ns[l], self.vmod[l], self.nmod[l], R, t, R_prev.T, t_prev, il,
                                         c.dist_thresh, c.angle_thresh)
                if sums[27] < 6:
                    ok = False
                    continue
                st, R2, t2, _ = orc.icp_solve(sums, R.ravel(), t)
                if st != 0:
                    ok = False
                    continue
                R, t = R2.reshape(3, 3), t2
        if ok:
            self.R, self.t = R, t
        return ok

    def process(self, depth):
        c = self.cfg
        ds, vs, ns = self.frame_maps(depth)
        ok = True
        if self.frames > 0:
            ok = self.track(vs, ns)
        self.lost.append(not ok)
        sd = orc.scale_depth_f64(depth, self.intr)
        orc.integrate_f64(sd, self.tsdf, self.weight, c.trunc_m, self.R.T, self.t, self.intr, self.cell64, self.rb,
                          c.max_weight)
        vm, nm = orc.raycast_f64(self.tsdf, self.rb, self.intr, self.R, self.t, c.trunc_m, self.cell64)
        self.vmod[0], self.nmod[0] = vm, nm
        for l in range(1, self.levels):
            # 2x2 means as the model pyramid, in FP64
            self.vmod[l] = _resize64(self.vmod[l - 1], False)
            self.nmod[l] = _resize64(self.nmod[l - 1], True)
        self.frames += 1
        return np.concatenate([self.R.ravel(), self.t])


def _resize64(m, normal):
    h, w, _ = m.shape
    b = m[: h // 2 * 2, : w // 2 * 2].reshape(h // 2, 2, w // 2, 2, 3)
    s = b.sum(axis=(1, 3))
    bad = np.isnan(b).any(axis=(1, 3, 4))
    if normal:
        s = s / np.linalg.norm(s, axis=-1, keepdims=True)
    else:
        s = s * 0.25
    s[bad] = np.nan
    return np.ascontiguousarray(s)
