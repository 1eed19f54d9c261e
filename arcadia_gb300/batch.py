"""Batched multi-view workload: several worlds x many views of mixed resolution in one launch.

``Batch`` owns one world slot per scene and device outputs per view, and fills the ``arc_view_desc``
table (layout.VIEW_DTYPE) for ``arc_trace_views_dev``. ``batched_config`` is the benchmark batch:
the 256^3, 512^3, 1024^3 and 1024^3-caves scenes, 16 views each, resolutions cycling from 320x240 to
2560x1440, camera poses drawn from a seeded generator inside each scene's bounds.
"""
from __future__ import annotations

import math

import numpy as np

from . import layout as L
from . import native

RESOLUTIONS = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (2560, 1440)]
BENCH_SCENES = ["c1_256", "s512", "s1024", "c2_1024_caves"]


def random_poses(scene: L.SceneParams, n: int, rng: np.random.Generator):
    """Eye positions inside the scene's bounds (upper part of the world, above most terrain),
    yaw uniform, pitch between -50 and -10 degrees."""
    ext = np.array(scene.grid, np.float64) * 16.0
    out = []
    for _ in range(n):
        eye = (rng.uniform(0.1, 0.9) * ext[0], rng.uniform(0.70, 0.95) * ext[1], rng.uniform(0.1, 0.9) * ext[2])
        out.append((eye, rng.uniform(0.0, 360.0), rng.uniform(-50.0, -10.0)))
    return out


class Batch:
    def __init__(self, tracer: native.Tracer, scenes, views_per_scene, resolutions=RESOLUTIONS, seed=2026,
                 quality=None, worlds=None):
        import torch

        self.t = tracer
        self.q = quality or L.quality_parity(512)
        self.views = []
        rng = np.random.default_rng(seed)
        pal = native.default_palette()
        self.buffers = []
        k = 0
        for slot, name in enumerate(scenes):
            scene = L.SCENES[name] if isinstance(name, str) else name
            if worlds is not None:
                roots, nodes, bricks = worlds[slot]
            else:
                roots, nodes, bricks, _ = native.build_world(scene)
            tracer.upload_world_slot(slot, scene.grid, roots, nodes, bricks, pal)
            for eye, yaw, pitch in random_poses(scene, views_per_scene, rng):
                w, h = resolutions[k % len(resolutions)]
                k += 1
                n = w * h
                bufs = [torch.zeros(m, dtype=torch.int32, device="cuda") for m in (n * 2, n * 2, n, n * 5, n * 5)]
                self.buffers.append(bufs)
                self.views.append(dict(slot=slot, scene=scene, w=w, h=h, eye=eye, yaw=yaw, pitch=pitch))
        self.table = np.zeros(len(self.views), L.VIEW_DTYPE)
        for i, (v, b) in enumerate(zip(self.views, self.buffers)):
            self.table[i]["world_slot"] = v["slot"]
            self.table[i]["width"] = v["w"]
            self.table[i]["height"] = v["h"]
            for f, buf in zip(("gbuf_depth_mat", "gbuf_norm_motion", "gbuf_albedo_ao", "hits", "gi_hits"), b):
                self.table[i][f] = buf.data_ptr()
        self.set_frame(0)

    @property
    def pixels(self) -> int:
        return int(sum(v["w"] * v["h"] for v in self.views))

    def camera(self, i, frame):
        v = self.views[i]
        return L.camera_uniforms(v["scene"].grid, v["w"], v["h"], v["eye"], yaw_deg=v["yaw"], pitch_deg=v["pitch"],
                                 quality=self.q, frame_index=frame)

    def set_frame(self, frame):
        for i in range(len(self.views)):
            self.table[i]["cam"] = self.camera(i, frame)[0]

    def trace(self, n_gi_ptr=0, use_graph=True):
        self.t.trace_views_dev(self.table, n_gi=n_gi_ptr, use_graph=use_graph)
