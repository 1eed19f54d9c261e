"""Radiance-cache comparison at secondary hits: neural radiance cache vs SHARC (the 1024^3 caves config).

Both caches learn the same quantity, the one-bounce radiance L(x) at the hit of each pixel's GI ray
(sun directional light with a shadow ray + constant sky through one cosine-sampled ray; see
``arc_onebounce_dev``), so the comparison is about the caching method alone:

  shared per frame  primary G-buffer (arc_trace_primary_dev) + GI hit points (arc_gi_points_dev),
                    which also compacts the pixels with a GI hit into a device list
  SHARC pipeline    arc_sharc_update_dev (tile-seeded paths, estimator deposits, mode 1) +
                    arc_sharc_resolve + arc_sharc_query_list_dev at every GI hit
  NRC pipeline      arc_nrc_train_frame_dev (one-bounce samples drawn from the list: 32,768 at the
                    operating point; fused forward/backward + Adam steps) + arc_nrc_query_list_dev at
                    every GI hit, or both in arc_nrc_frame_dev (the query beside the sample generation)

Neither pipeline reads anything back to the host during a frame.

The surfaces are Lambertian with one albedo per material (U[0.1, 0.9] per channel). SHARC caches the
reflected radiance as the reference does. The network learns the demodulated quantity L / albedo,
which depends only on position and normal (the inputs it is given), and the query multiplies the
albedo back in.

Quality is the relative MSE, mean((pred - ref)^2 / (ref^2 + 0.01)), against a 4096-spp reference of
the estimator at a fixed set of GI hit points. The reference is traced in FP32 on the GPU (64
launches of 64 spp) and accumulated in FP64 on the host.
"""
from __future__ import annotations

import ctypes as C
import statistics

import numpy as np

from . import layout as L
from . import native

TRAIN_SAMPLES = 65536
# Adam learning rate of the cache comparison and the pipeline. Measured on 300 static 1080p frames of the
# 1024^3 caves world (32,768 samples x 4 steps per frame): with 1e-2 the network is below SHARC at every
# scored frame from 10 on; with 1e-3 its error rises between frames 30 and 120 before falling again.
LEARNING_RATE = 1e-2
REF_SPP_PER_LAUNCH = 64
REF_LAUNCHES = 64


def rel_mse(pred: np.ndarray, ref: np.ndarray) -> float:
    pred = pred.astype(np.float64)
    return float(np.mean((pred - ref) ** 2 / (ref ** 2 + 0.01)))


class CacheComparison:
    def __init__(self, tracer: native.Tracer, scene: L.SceneParams, width: int, height: int, quality=None):
        import torch

        self.torch = torch
        self.t = tracer
        self.scene = scene
        self.w, self.h = width, height
        self.q = quality or L.quality_high()
        n = width * height
        dev = torch.device("cuda")
        i32 = torch.int32
        self.gdm = torch.empty(n * 2, dtype=i32, device=dev)
        self.gnm = torch.empty(n * 2, dtype=i32, device=dev)
        self.gaa = torch.empty(n, dtype=i32, device=dev)
        self.pos = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        self.nrm = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        self.alb = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        self.nin = torch.zeros((n, 9), dtype=torch.float32, device=dev)
        self.valid = torch.zeros(n, dtype=i32, device=dev)
        self.n_valid = torch.zeros(1, dtype=torch.int64, device=dev)
        self.list = torch.zeros(n, dtype=i32, device=dev)
        self.sharc_out = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        self.nrc_out = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        self.stream = torch.cuda.ExternalStream(tracer.stream())
        self.lib = native.lib()

    def camera(self, frame):
        return L.default_camera_for(self.scene, self.w, self.h, quality=self.q, frame_index=frame)

    def _ck(self, rc, what):
        if rc:
            raise native.ArcError(rc, f"{what}: {self.t.last_error()}")

    def _event(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e

    def shared(self, frame):
        """Primary pass + GI hit points of `frame`; returns its device time in ms."""
        self.t.set_camera(self.camera(frame))
        a = self._event()
        self.t.trace_primary_dev(self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr(), self.gaa.data_ptr())
        self._ck(self.lib.arc_gi_points_dev(self.t.ctx, self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr(),
                                            self.pos.data_ptr(), self.nrm.data_ptr(), self.alb.data_ptr(),
                                            self.nin.data_ptr(), self.valid.data_ptr(), self.n_valid.data_ptr(),
                                            self.list.data_ptr()), "arc_gi_points_dev")
        b = self._event()
        b.synchronize()
        return a.elapsed_time(b)

    def sharc_frame(self, overlap=False):
        """SHARC update + resolve + query at every GI hit; with overlap the query runs beside the update
        against the previous frame's resolve (arc_sharc_frame_dev). Returns its device time in ms."""
        a = self._event()
        if overlap:
            self._ck(self.lib.arc_sharc_frame_dev(self.t.ctx, self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr(),
                                                  self.list.data_ptr(), self.n_valid.data_ptr(), self.w * self.h,
                                                  self.pos.data_ptr(), self.nrm.data_ptr(), self.sharc_out.data_ptr()),
                     "arc_sharc_frame_dev")
        else:
            self._ck(self.lib.arc_sharc_update_dev(self.t.ctx, self.w, self.h, self.gdm.data_ptr(), self.gnm.data_ptr()),
                     "arc_sharc_update_dev")
            self._ck(self.lib.arc_sharc_resolve(self.t.ctx), "arc_sharc_resolve")
            self._ck(self.lib.arc_sharc_query_list_dev(self.t.ctx, self.list.data_ptr(), self.n_valid.data_ptr(),
                                                       self.w * self.h, self.pos.data_ptr(), self.nrm.data_ptr(),
                                                       self.sharc_out.data_ptr()), "arc_sharc_query_list_dev")
        b = self._event()
        b.synchronize()
        return a.elapsed_time(b)

    def nrc_frame(self, seed, lr=LEARNING_RATE, steps=8, overlap=False, samples=TRAIN_SAMPLES):
        """One training frame (TRAIN_SAMPLES samples, `steps` Adam steps on equal slices) and inference at
        every GI hit; with overlap the inference runs beside the sample generation with the previous
        frame's weights (arc_nrc_frame_dev). Returns its device time in ms."""
        a = self._event()
        if overlap:
            self._ck(self.lib.arc_nrc_frame_dev(self.t.ctx, self.list.data_ptr(), self.n_valid.data_ptr(), self.w * self.h,
                                                self.pos.data_ptr(), self.nrm.data_ptr(), self.nin.data_ptr(),
                                                self.alb.data_ptr(), self.nrc_out.data_ptr(), seed, samples, steps,
                                                C.c_float(lr)), "arc_nrc_frame_dev")
        else:
            self._ck(self.lib.arc_nrc_train_frame_dev(self.t.ctx, self.list.data_ptr(), self.n_valid.data_ptr(),
                                                      self.pos.data_ptr(), self.nrm.data_ptr(), self.nin.data_ptr(), seed,
                                                      samples, steps, C.c_float(lr)), "arc_nrc_train_frame_dev")
            self._ck(self.lib.arc_nrc_query_list_dev(self.t.ctx, self.list.data_ptr(), self.n_valid.data_ptr(),
                                                     self.w * self.h, self.nin.data_ptr(), self.alb.data_ptr(),
                                                     self.nrc_out.data_ptr()), "arc_nrc_query_list_dev")
        b = self._event()
        b.synchronize()
        return a.elapsed_time(b)

    def reference(self, idx: np.ndarray, seed=12345):
        """4096-spp one-bounce reference at pixels idx (FP32 launches, FP64 host accumulation)."""
        torch = self.torch
        d_idx = torch.from_numpy(idx.astype(np.int32)).cuda()
        out = torch.zeros((len(idx), 3), dtype=torch.float32, device="cuda")
        acc = np.zeros((len(idx), 3), np.float64)
        for k in range(REF_LAUNCHES):
            self._ck(self.lib.arc_onebounce_dev(self.t.ctx, d_idx.data_ptr(), len(idx), self.pos.data_ptr(),
                                                self.nrm.data_ptr(), self.alb.data_ptr(), REF_SPP_PER_LAUNCH,
                                                seed + 7919 * k, 0, out.data_ptr()), "arc_onebounce_dev")
            torch.cuda.synchronize()
            acc += out.cpu().numpy().astype(np.float64)
        return acc / REF_LAUNCHES

    def one_sample(self, idx: np.ndarray, seed=999):
        """1-spp estimate at pixels idx: the method without any cache."""
        torch = self.torch
        d_idx = torch.from_numpy(idx.astype(np.int32)).cuda()
        out = torch.zeros((len(idx), 3), dtype=torch.float32, device="cuda")
        self._ck(self.lib.arc_onebounce_dev(self.t.ctx, d_idx.data_ptr(), len(idx), self.pos.data_ptr(),
                                            self.nrm.data_ptr(), self.alb.data_ptr(), 1, seed, 0, out.data_ptr()),
                 "arc_onebounce_dev")
        torch.cuda.synchronize()
        return out.cpu().numpy()


def run_comparison(tracer: native.Tracer, scene_name="c2_1024_caves", width=1920, height=1080, frames=300,
                   eval_points=16384, seed=7, steps_per_frame=8, lr=LEARNING_RATE, curve=(30, 60, 120), overlap=False,
                   train_samples=TRAIN_SAMPLES, boost_frames=0, boost_steps=16, lr_warmup_frames=0):
    """Runs both pipelines for `frames` frames on a static camera and scores them on the last frame;
    `curve` lists earlier frames at which both are scored as well (8192 points each). With overlap each
    cache's query runs beside its own update (one frame behind it), for both caches alike. The first
    `boost_frames` frames train with `boost_steps` Adam steps instead of `steps_per_frame` (a start-up
    phase; the timings average the second half of the run). With lr_warmup_frames the learning rate
    rises linearly to `lr` over that many frames."""
    scene = L.SCENES[scene_name]
    cc = CacheComparison(tracer, scene, width, height)
    lib = cc.lib
    cc._ck(lib.arc_sharc_set_mode(tracer.ctx, 1), "arc_sharc_set_mode")
    tracer.sharc_reset()
    cc._ck(lib.arc_nrc_init(tracer.ctx, seed), "arc_nrc_init")
    shared_ms, sharc_ms, nrc_ms = [], [], []
    conv = []
    for f in range(frames):
        shared_ms.append(cc.shared(f))
        sharc_ms.append(cc.sharc_frame(overlap=overlap))
        steps = boost_steps if f < boost_frames else steps_per_frame
        lr_f = lr * min(1.0, (f + 1) / lr_warmup_frames) if lr_warmup_frames else lr
        nrc_ms.append(cc.nrc_frame(seed * 1000003 + f, lr=lr_f, steps=steps, overlap=overlap, samples=train_samples))
        if f + 1 in curve and f + 1 < frames:
            cand = np.nonzero(cc.valid.cpu().numpy().astype(bool))[0]
            ci = cand[np.linspace(0, len(cand) - 1, min(8192, len(cand))).astype(np.int64)]
            cref = cc.reference(ci)
            conv.append({"frame": f + 1, "rel_mse_nrc": rel_mse(cc.nrc_out.cpu().numpy()[ci], cref),
                         "rel_mse_sharc": rel_mse(cc.sharc_out.cpu().numpy()[ci][:, :3], cref)})
    valid = cc.valid.cpu().numpy().astype(bool)
    cand = np.nonzero(valid)[0]
    idx = cand[np.linspace(0, len(cand) - 1, min(eval_points, len(cand))).astype(np.int64)]
    ref = cc.reference(idx)
    sharc = cc.sharc_out.cpu().numpy()[idx]
    nrc = cc.nrc_out.cpu().numpy()[idx]
    raw = cc.one_sample(idx)
    sharc_hit = sharc[:, 3] > 0.5
    # untrained network, same points (the method without the learned part)
    cc._ck(lib.arc_nrc_init(tracer.ctx, seed), "arc_nrc_init")
    cc._ck(lib.arc_nrc_query_list_dev(tracer.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), width * height,
                                      cc.nin.data_ptr(), cc.alb.data_ptr(), cc.nrc_out.data_ptr()), "query")
    tracer.synchronize()
    untrained = cc.nrc_out.cpu().numpy()[idx]
    cc._ck(lib.arc_sharc_set_mode(tracer.ctx, 0), "arc_sharc_set_mode")
    steady = slice(frames // 2, None)
    return {
        "frames": frames,
        "overlap": overlap,
        "train_samples": train_samples,
        "train_steps_per_frame": steps_per_frame,
        "boost_frames": boost_frames,
        "lr": lr,
        "width": width,
        "height": height,
        "eval_points": int(len(idx)),
        "reference_spp": REF_SPP_PER_LAUNCH * REF_LAUNCHES,
        "shared_ms_per_frame": round(statistics.mean(shared_ms[steady]), 4),
        "nrc_cache_ms_per_frame": round(statistics.mean(nrc_ms[steady]), 4),
        "sharc_cache_ms_per_frame": round(statistics.mean(sharc_ms[steady]), 4),
        "nrc_ms_per_frame": round(statistics.mean(shared_ms[steady]) + statistics.mean(nrc_ms[steady]), 4),
        "sharc_ms_per_frame": round(statistics.mean(shared_ms[steady]) + statistics.mean(sharc_ms[steady]), 4),
        "rel_mse_nrc": rel_mse(nrc, ref),
        "rel_mse_sharc": rel_mse(sharc[:, :3], ref),
        "sharc_hit_fraction": float(sharc_hit.mean()),
        "rel_mse_sharc_on_hits": rel_mse(sharc[sharc_hit, :3], ref[sharc_hit]) if sharc_hit.any() else None,
        "rel_mse_nrc_on_sharc_hits": rel_mse(nrc[sharc_hit], ref[sharc_hit]) if sharc_hit.any() else None,
        "rel_mse_1spp": rel_mse(raw, ref),
        "rel_mse_untrained_nrc": rel_mse(untrained, ref),
        "convergence": conv,
    }


NRC_FLOPS_PER_QUERY = 2 * (216 * 64 + 4 * 64 * 64 + 3 * 64)  # 60,800


def kernel_timing(tracer: native.Tracer, scene_name="c2_1024_caves", width=1920, height=1080, reps=5):
    """Device times (CUDA events, median of reps) of the NRC stages on one frame's GI hits, for the
    tcgen05 kernels and the mma.sync kernels: inference over the hit list, one training frame with
    1 Adam step, and the extra cost of each further step."""
    import torch

    scene = L.SCENES[scene_name]
    cc = CacheComparison(tracer, scene, width, height)
    cc.shared(5)
    lib = cc.lib
    cc._ck(lib.arc_nrc_init(tracer.ctx, 3), "arc_nrc_init")
    n_px = width * height
    n_hits = int(cc.n_valid.item())

    def timed(fn):
        ms = []
        for _ in range(reps):
            a = cc._event()
            fn()
            b = cc._event()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return statistics.median(ms)

    def query():
        cc._ck(lib.arc_nrc_query_list_dev(tracer.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), n_px, cc.nin.data_ptr(),
                                          cc.alb.data_ptr(), cc.nrc_out.data_ptr()), "query")

    def train(steps):
        return lambda: cc._ck(lib.arc_nrc_train_frame_dev(tracer.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(),
                                                          cc.pos.data_ptr(), cc.nrm.data_ptr(), cc.nin.data_ptr(), 9,
                                                          TRAIN_SAMPLES, steps, C.c_float(1e-3)), "train")

    out = {"gi_hits": n_hits, "train_samples": TRAIN_SAMPLES, "flops_per_query": NRC_FLOPS_PER_QUERY}
    # tcgen05 inference with one tile group per CTA (the default, two CTAs per SM), with four groups in
    # one CTA per SM, and the mma.sync kernels
    for name, path in (("tcgen05", 1), ("tcgen05_four_groups", 2), ("mma_sync", 0)):
        cc._ck(lib.arc_nrc_set_infer_path(tracer.ctx, path), "path")
        cc._ck(lib.arc_nrc_set_train_path(tracer.ctx, min(path, 1)), "path")
        q = timed(query)
        t1, t8 = timed(train(1)), timed(train(8))
        out[name] = {"query_ms": round(q, 4), "query_tflops": round(n_hits * NRC_FLOPS_PER_QUERY / (q * 1e-3) / 1e12, 1),
                     "train_frame_1step_ms": round(t1, 4), "per_extra_step_ms": round((t8 - t1) / 7, 4)}
    cc._ck(lib.arc_nrc_set_infer_path(tracer.ctx, 3), "path")
    cc._ck(lib.arc_nrc_set_train_path(tracer.ctx, 1), "path")
    return out
