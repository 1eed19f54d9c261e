"""Full per-frame pipeline over an editable world: in-place edits, primary + GI trace, NRC at the
secondary hits.

Per frame ``FullPipeline.frame`` runs, in stream order on the tracer's stream:
  edits    a seeded batch of carves and recolours aimed at surfaces the previous frame hit
           (``edits.batch_from_hits``), sized so that about ``edit_fraction`` of the world's leaf
           bricks are rewritten per frame (``arc_apply_edits``: the tree is updated in place before
           traversal)
  trace    ``arc_trace_frame_dev``: primary G-buffer + hit records + one GI ray per hit pixel
  points   ``arc_gi_points_from_hits_dev``: NRC inputs at the GI hits from the hit records
  nrc      ``arc_nrc_train_frame_dev`` (online training) + ``arc_nrc_query_list_dev`` at every GI hit
Each stage is timed with CUDA events. The camera follows a seeded circular path above the terrain.
The edit batches are kept (``ops_log``) so that a test can replay them on the oracle.

With ``compare_every`` > 0 the SHARC pipeline runs beside the NRC on the same frames, after the timed
stages (update in mode 1 from this frame's G-buffer, resolve, query at the same GI hit list), and every
``compare_every`` frames both caches are scored against a 4096-spp reference of the one-bounce
estimator at 4096 of the frame's GI hits (rel-MSE, as in the static cache comparison): how each cache
keeps up with a moving camera over a world that is edited every frame.
"""
from __future__ import annotations

import ctypes as C
import math
import statistics

import numpy as np

from . import layout as L
from . import native
from .edits import batch_from_hits, ops_for_brick_budget
from .gi_cache import LEARNING_RATE

TRAIN_SAMPLES = 32768  # the cache comparison's operating point (with 4 Adam steps per frame)


def path_camera(scene: L.SceneParams, width: int, height: int, frame: int, n_frames: int, quality=None):
    """Circular path around the world centre, 30 % of the world's width out, above the highest
    terrain (height_hi + 8 % of the world height), looking 32 degrees down, 20 degrees inward."""
    gx, gy, gz = scene.grid
    ext = np.array([gx, gy, gz], np.float64) * 16.0  # metres
    a = 2.0 * math.pi * frame / max(n_frames, 1)
    eye = (ext[0] * (0.5 + 0.3 * math.cos(a)), ext[1] * min(scene.height_hi + 0.08, 0.95), ext[2] * (0.5 + 0.3 * math.sin(a)))
    yaw = math.degrees(a) + 180.0 + 20.0  # tangent of the circle, turned towards the centre
    return L.camera_uniforms(scene.grid, width, height, eye, yaw_deg=yaw, pitch_deg=-32.0, quality=quality,
                             frame_index=frame)


class FullPipeline:
    def __init__(self, tracer: native.Tracer, scene: L.SceneParams, width: int, height: int, n_bricks: int,
                 n_frames: int = 300, edit_fraction: float = 0.01, nrc_steps: int = 4, seed: int = 2027, quality=None,
                 keep_ops: bool = False, compare_every: int = 0, compare_points: int = 4096, boost_frames: int = 0,
                 boost_steps: int = 16, lr_warmup_frames: int = 0, lr: float | None = None,
                 train_samples: int = TRAIN_SAMPLES):
        import torch

        self.torch = torch
        self.t = tracer
        self.scene = scene
        self.w, self.h = width, height
        self.n_frames = n_frames
        self.q = quality or L.quality_high()
        self.nrc_steps = nrc_steps
        self.boost_frames, self.boost_steps = boost_frames, boost_steps
        self.lr_warmup_frames = lr_warmup_frames
        self.lr = LEARNING_RATE if lr is None else lr
        self.train_samples = train_samples
        self.rng = np.random.default_rng(seed)
        self.seed = seed
        self.brick_target = max(1, int(round(edit_fraction * n_bricks)))
        self.bricks_per_op = 30.0  # first guess; refined from the measured counts
        self.keep_ops = keep_ops
        self.ops_log = []
        n = width * height
        dev = torch.device("cuda")
        i32, f32 = torch.int32, torch.float32
        self.gdm = torch.zeros(2 * n, dtype=i32, device=dev)
        self.gnm = torch.zeros(2 * n, dtype=i32, device=dev)
        self.gaa = torch.zeros(n, dtype=i32, device=dev)
        self.hits = torch.zeros(5 * n, dtype=i32, device=dev)
        self.gi = torch.zeros(5 * n, dtype=i32, device=dev)
        self.n_gi = torch.zeros(1, dtype=torch.int64, device=dev)
        self.pos = torch.zeros((n, 3), dtype=f32, device=dev)
        self.nrm = torch.zeros((n, 3), dtype=f32, device=dev)
        self.alb = torch.zeros((n, 3), dtype=f32, device=dev)
        self.nin = torch.zeros((n, 9), dtype=f32, device=dev)
        self.valid = torch.zeros(n, dtype=i32, device=dev)
        self.n_valid = torch.zeros(1, dtype=torch.int64, device=dev)
        self.list = torch.zeros(n, dtype=i32, device=dev)
        self.nrc_out = torch.zeros((n, 3), dtype=f32, device=dev)
        self.stream = torch.cuda.ExternalStream(tracer.stream())
        self.lib = native.lib()
        self._ck(self.lib.arc_nrc_init(tracer.ctx, seed), "arc_nrc_init")
        self.last_rewritten = tracer.edit_stats()["bricks_rewritten"]
        self.records = []
        self.launch = None
        self.compare_every = compare_every
        self.compare_points = compare_points
        self.path_scores = []
        if compare_every:
            self.sharc_out = torch.zeros((n, 4), dtype=f32, device=dev)
            self._ck(self.lib.arc_sharc_set_mode(tracer.ctx, 1), "arc_sharc_set_mode")
            self._ck(self.lib.arc_sharc_reset(tracer.ctx), "arc_sharc_reset")

    def _ck(self, rc, what):
        if rc:
            raise native.ArcError(rc, f"{what}: {self.t.last_error()}")

    def _event(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e

    def _edit_batch(self):
        """Edits at hit points of the previous frame, sized to the brick budget."""
        n_ops = ops_for_brick_budget(self.brick_target, self.bricks_per_op)
        n_px = self.w * self.h
        idx = self.torch.from_numpy(self.rng.integers(0, n_px, 4 * n_ops)).cuda()
        rows = self.hits.view(n_px, 5)[idx].cpu().numpy().view(L.HIT_DTYPE).reshape(-1)
        return batch_from_hits(rows, n_ops, self.rng)

    def frame(self, f: int):
        torch = self.torch
        ops = self._edit_batch() if f > 0 else np.zeros(0, L.EDIT_DTYPE)
        if self.keep_ops:
            self.ops_log.append(ops.copy())
        e0 = self._event()
        if len(ops):
            self.t.apply_edits(ops)
        e1 = self._event()
        self.t.set_camera(path_camera(self.scene, self.w, self.h, f, self.n_frames, self.q))
        self.t.trace_frame_dev(self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr(), self.gaa.data_ptr(),
                               self.hits.data_ptr(), self.gi.data_ptr(), self.n_gi.data_ptr())
        e2 = self._event()
        self._ck(self.lib.arc_gi_points_from_hits_dev(self.t.ctx, self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr(),
                                                      self.gi.data_ptr(), self.pos.data_ptr(), self.nrm.data_ptr(),
                                                      self.alb.data_ptr(), self.nin.data_ptr(), self.valid.data_ptr(),
                                                      self.n_valid.data_ptr(), self.list.data_ptr()),
                 "arc_gi_points_from_hits_dev")
        e3 = self._event()
        n_px = self.w * self.h
        self._ck(self.lib.arc_nrc_train_frame_dev(self.t.ctx, self.list.data_ptr(), self.n_valid.data_ptr(),
                                                  self.pos.data_ptr(), self.nrm.data_ptr(), self.nin.data_ptr(),
                                                  self.seed * 7919 + f, self.train_samples,
                                                  self.boost_steps if f < self.boost_frames else self.nrc_steps,
                                                  C.c_float(self.lr * min(1.0, (f + 1) / self.lr_warmup_frames)
                                                            if self.lr_warmup_frames else self.lr)),
                 "arc_nrc_train_frame_dev")
        self._ck(self.lib.arc_nrc_query_list_dev(self.t.ctx, self.list.data_ptr(), self.n_valid.data_ptr(), n_px,
                                                 self.nin.data_ptr(), self.alb.data_ptr(), self.nrc_out.data_ptr()),
                 "arc_nrc_query_list_dev")
        e4 = self._event()
        e5 = None
        if self.compare_every:  # SHARC beside the NRC, timed on its own after the frame's NRC work
            self._sharc_frame()
            e5 = self._event()
        (e5 or e4).synchronize()
        rewritten = self.t.edit_stats()["bricks_rewritten"]
        dr = rewritten - self.last_rewritten
        self.last_rewritten = rewritten
        if len(ops) and dr > 0:
            self.bricks_per_op = 0.7 * self.bricks_per_op + 0.3 * (dr / len(ops))
        rec = {"edit_ms": e0.elapsed_time(e1), "trace_ms": e1.elapsed_time(e2), "points_ms": e2.elapsed_time(e3),
               "nrc_ms": e3.elapsed_time(e4), "total_ms": e0.elapsed_time(e4), "ops": int(len(ops)),
               "sharc_ms": e4.elapsed_time(e5) if e5 is not None else None,
               "bricks_rewritten": int(dr), "rays": n_px + int(self.n_gi.item()), "gi_hits": int(self.n_valid.item())}
        self.records.append(rec)
        if self.compare_every and (f + 1) % self.compare_every == 0:
            self.path_scores.append(self._score(f))
        return rec

    def _sharc_frame(self):
        """SHARC beside the NRC (timed on its own, outside the frame's total): mode-1 update from this
        frame's G-buffer, resolve, query at the frame's GI hit list."""
        n_px = self.w * self.h
        self._ck(self.lib.arc_sharc_update_dev(self.t.ctx, self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr()),
                 "arc_sharc_update_dev")
        self._ck(self.lib.arc_sharc_resolve(self.t.ctx), "arc_sharc_resolve")
        self._ck(self.lib.arc_sharc_query_list_dev(self.t.ctx, self.list.data_ptr(), self.n_valid.data_ptr(), n_px,
                                                   self.pos.data_ptr(), self.nrm.data_ptr(), self.sharc_out.data_ptr()),
                 "arc_sharc_query_list_dev")

    def _score(self, f: int):
        """rel-MSE of both caches at `compare_points` of this frame's GI hits against 64 x 64 spp of the
        estimator (FP32 launches, FP64 accumulation on the host)."""
        from .gi_cache import REF_LAUNCHES, REF_SPP_PER_LAUNCH, rel_mse

        torch = self.torch
        self.t.synchronize()
        cand = np.nonzero(self.valid.cpu().numpy().astype(bool))[0]
        idx = cand[np.linspace(0, len(cand) - 1, min(self.compare_points, len(cand))).astype(np.int64)]
        d_idx = torch.from_numpy(idx.astype(np.int32)).cuda()
        out = torch.zeros((len(idx), 3), dtype=torch.float32, device="cuda")
        acc = np.zeros((len(idx), 3), np.float64)
        for k in range(REF_LAUNCHES):
            self._ck(self.lib.arc_onebounce_dev(self.t.ctx, d_idx.data_ptr(), len(idx), self.pos.data_ptr(),
                                                self.nrm.data_ptr(), self.alb.data_ptr(), REF_SPP_PER_LAUNCH,
                                                777 + 7919 * k + 104729 * f, 0, out.data_ptr()), "arc_onebounce_dev")
            self.t.synchronize()
            acc += out.cpu().numpy().astype(np.float64)
        ref = acc / REF_LAUNCHES
        nrc = self.nrc_out.cpu().numpy()[idx]
        sharc = self.sharc_out.cpu().numpy()[idx, :3]
        return {"frame": f + 1, "rel_mse_nrc": round(rel_mse(nrc, ref), 4), "rel_mse_sharc": round(rel_mse(sharc, ref), 4)}

    def tune(self):
        """Untimed setup: the frame autotuner picks the launch configuration on the path's first view."""
        self.t.set_camera(path_camera(self.scene, self.w, self.h, 0, self.n_frames, self.q))
        best, ms = self.t.autotune_frame_dev(self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr(), self.gaa.data_ptr(),
                                             self.hits.data_ptr(), self.gi.data_ptr(), frames=2)
        self.launch = {"kernel": "persistent" if best.variant == 1 else "plain", "block_threads": best.block_threads,
                       "reg_blocks": best.reg_blocks, "tuned_ms": round(ms, 4)}

    def run(self, warmup: int = 3, autotune: bool = True):
        if autotune:
            self.tune()
        for f in range(self.n_frames):
            self.frame(f)
        return self.summary(warmup)

    def summary(self, skip: int = 3):
        r = self.records[skip:] if len(self.records) > skip else self.records
        med = lambda k: round(statistics.median(x[k] for x in r), 4)
        trace_ms = sum(x["trace_ms"] for x in r)
        total_ms = sum(x["total_ms"] for x in r)
        rays = sum(x["rays"] for x in r)
        st = self.t.edit_stats()
        return {
            "frames": len(self.records), "frames_summarised": len(r), "width": self.w, "height": self.h,
            "ms_per_frame": round(total_ms / len(r), 4), "median_ms": {k: med(k) for k in
                                                                      ("edit_ms", "trace_ms", "points_ms", "nrc_ms", "total_ms")},
            **({"sharc_ms_median": med("sharc_ms")} if self.compare_every else {}),
            "trace_mrays_per_s": round(rays / (trace_ms * 1e-3) / 1e6, 2),
            "pipeline_mrays_per_s": round(rays / (total_ms * 1e-3) / 1e6, 2),
            "edit_ops_per_frame": round(statistics.mean(x["ops"] for x in r), 1),
            "bricks_rewritten_per_frame": round(statistics.mean(x["bricks_rewritten"] for x in r), 1),
            "brick_target_per_frame": self.brick_target,
            "gi_hits_per_frame": round(statistics.mean(x["gi_hits"] for x in r), 1),
            "nrc_train_samples": self.train_samples, "nrc_steps": self.nrc_steps,
            "pool_next_node": st["next_node"], "pool_next_brick": st["next_brick"], "overflow": st["overflow"],
            "device_status": self.t.stats().device_status, "launch": self.launch,
            **({"cache_scores_along_path": self.path_scores} if self.compare_every else {}),
        }
