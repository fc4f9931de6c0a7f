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
