"""Multi-scene serving: continuous batching of ray chunks under CUDA graphs.

Pieces:

* ``ChunkPipeline`` renders one chunk of `chunk_rays` pixels of a frame with the served chain, from fixed
  device buffers and with no host synchronisation:
  1. pinhole rays from camera parameters in device memory (`nsvf_pinhole_rays`);
  2. SVO intersection + depth sort (`nsvf_svo_intersect_sorted`);
  3. order-preserving hit compaction (torch cumsum + `nsvf_compact_hits`);
  4. the hit rays' lists and sampling distribution (`nsvf_gather_probs`);
  5. inverse-CDF sample count, offsets (torch cumsum) and compaction (`nsvf_sample_count_dev`,
     `nsvf_sample_compact_dev`), with the reference wrapper's launch layout taken from the device-side hit
     count;
  6. interpolation + tcgen05 BF16 MLP on the device-side sample count (`nsvf_field_samples_bf16_dev`),
     then the double-float re-evaluation of the samples far outside their voxel (`nsvf_field_exact_dev`)
     and the FP32 re-evaluation of the rays where such a sample's colour is large
     (`nsvf_field_refine_fp32_dev`);
  7. compensated compositing + background into the chunk's output (`nsvf_composite_segments_dev`).

  It is captured once into a CUDA graph and replayed per chunk. The only per-chunk input is 18 camera
  floats, including the chunk's first pixel and pixel count, copied into the pipeline's parameter buffer
  before the replay.
* ``SceneStore`` holds resident scenes (`SceneState`), counted against an HBM budget.
* ``Server`` is the request loop:
  - A request (scene, camera, resolution) is admitted when an in-flight slot and enough of the frame-buffer
    budget are free.
  - Every free pipeline slot takes the next chunk of the oldest admitted frame. Chunks of frames of
    different scenes and resolutions therefore run on the GPU at the same time, on separate streams.
  - A frame completes when all its chunks are composited and copied to its pinned host buffer. Its latency
    is completion minus arrival.

A pipeline holds at most `chunk_rays * samples_per_ray` samples. A chunk that needs more sets bit 1 of its
error word (bit 4 for more far-outside samples than its list holds); the server then renders that chunk again with the synchronising served path (`render_frame`),
so results never depend on the capacity.
"""
import math
import time
from collections import deque

import numpy as np
import torch

from . import scenes
from ._lib import LIB, check
from .served import REFINE_ABOVE, SceneState, render_frame


def _p(t):
    return t.data_ptr() if t is not None else None


def camera_params(cam, width, height, focal, first=0, count=None):
    """18 floats: origin, camera-to-world rotation (row-major), focal, cx, cy,
    width, first pixel, pixel count (see nsvf_pinhole_rays)."""
    R = scenes.look_at(np.asarray(cam, np.float64))
    out = np.zeros(18, np.float32)
    out[0:3] = cam
    out[3:12] = R.reshape(-1)
    out[12] = focal
    out[13] = width / 2.0
    out[14] = height / 2.0
    out[15] = width
    out[16] = first
    out[17] = width * height - first if count is None else count
    return out


class ChunkPipeline:
    """Fixed-size, synchronisation-free render of one ray chunk of one scene."""

    def __init__(self, scene, chunk_rays, samples_per_ray=256, stream=None, use_graph=True):
        self.scene = scene
        self.C = int(chunk_rays)
        self.cap = int(chunk_rays) * int(samples_per_ray)
        dev = scene.device
        self.device = dev
        self.stream = stream if stream is not None else torch.cuda.Stream(dev)
        C, H = self.C, scene.max_hits
        i32, f32, i64, u8 = torch.int32, torch.float32, torch.int64, torch.uint8

        def z(*s, dtype=f32):
            return torch.zeros(*s, dtype=dtype, device=dev)

        self.cam = z(18)
        self.cam_host = torch.zeros(18, dtype=f32).pin_memory()
        self.ro, self.rd = z(C, 3), z(C, 3)
        self.idx, self.lo, self.hi = z(C, H, dtype=i32), z(C, H), z(C, H)
        self.hits = z(C, dtype=u8)
        self.scan = z(C, dtype=i32)
        self.pix = z(C, dtype=i64)
        self.n_hit = z(1, dtype=i64)
        self.I, self.L, self.U = z(C, H, dtype=i32), z(C, H), z(C, H)
        self.probs, self.steps = z(C, H), z(C)
        self.count = z(C, dtype=i32)
        self.offset = z(C + 1, dtype=i64)
        self.vox = z(self.cap, dtype=i32)
        self.xyzd = z(self.cap, 4)
        self.sdepth = z(self.cap)
        self.field = z(self.cap, 4)
        self.colors, self.depths, self.missed = z(C, 3), z(C), z(C)
        self.err = z(1, dtype=i32)
        # samples far outside their voxel, re-evaluated in double-float
        self.outl_cap = max(4096, self.cap // 1024)
        self.outl = z(self.outl_cap, dtype=i64)
        self.n_outl = z(1, dtype=i64)
        # rays re-evaluated in FP32 (their far-outside sample's colour is large)
        self.refine_rows = z(self.outl_cap, dtype=i64)
        self.n_refine = z(1, dtype=i64)
        n_nodes = scene.octree_centers.shape[0]
        self.ws = torch.empty(max(16, int(LIB.nsvf_svo_workspace_bytes(1, n_nodes))), dtype=u8,
                              device=dev)
        self.bg = torch.tensor(list(scene.bg), device=dev)
        self.graph = None
        self.use_graph = use_graph

    def _enqueue(self):
        sc, C, H, s = self.scene, self.C, self.scene.max_hits, self.stream.cuda_stream
        check(LIB.nsvf_pinhole_rays(C, _p(self.cam), _p(self.ro), _p(self.rd), s), "pinhole_rays")
        check(LIB.nsvf_svo_intersect_sorted(1, 1, sc.octree_centers.shape[0], C, sc.voxel_size, H,
                                            _p(self.ro), _p(self.rd), _p(sc.octree_centers),
                                            _p(sc.octree_children), _p(self.idx), _p(self.lo),
                                            _p(self.hi), _p(self.hits), _p(self.err), _p(self.ws),
                                            s), "svo_intersect_sorted")
        torch.cumsum(self.hits, 0, dtype=torch.int32, out=self.scan)
        check(LIB.nsvf_compact_hits(C, _p(self.hits), _p(self.scan), _p(self.pix), _p(self.n_hit),
                                    s), "compact_hits")
        check(LIB.nsvf_gather_probs(C, _p(self.n_hit), H, sc.step_size, _p(self.pix), _p(self.idx),
                                    _p(self.lo), _p(self.hi), _p(self.I), _p(self.L), _p(self.U),
                                    _p(self.probs), _p(self.steps), s), "gather_probs")
        check(LIB.nsvf_sample_count_dev(C, _p(self.n_hit), H, _p(self.I), _p(self.L), _p(self.U),
                                        _p(self.probs), _p(self.steps), _p(self.count), s),
              "sample_count_dev")
        torch.cumsum(self.count, 0, out=self.offset[1:])
        check(LIB.nsvf_sample_compact_dev(C, _p(self.n_hit), H, _p(self.I), _p(self.L),
                                          _p(self.U), _p(self.probs), _p(self.steps), _p(self.ro),
                                          3, _p(self.rd), _p(self.pix), _p(self.offset), self.cap,
                                          _p(self.vox), _p(self.xyzd), _p(self.sdepth),
                                          _p(self.err), s), "sample_compact_dev")
        m = sc.mlp
        self.n_outl.zero_()
        self.n_refine.zero_()
        check(LIB.nsvf_field_samples_bf16_dev(self.cap, _p(self.offset[C:]), _p(self.vox),
                                              _p(self.xyzd), sc.centers.size(0), sc.values.size(0),
                                              sc.voxel_size, _p(sc.centers), _p(sc.feats),
                                              _p(sc.values), m._wp, m._bp_tc, _p(self.field),
                                              _p(self.outl), _p(self.n_outl), self.outl_cap,
                                              _p(self.err), s), "field_samples_bf16_dev")
        check(LIB.nsvf_field_exact_dev(C, _p(self.n_hit), _p(self.offset), _p(self.pix),
                                       _p(self.ro), 3, _p(self.rd), _p(self.sdepth), _p(self.vox),
                                       sc.centers.size(0), sc.values.size(0), sc.voxel_size,
                                       _p(sc.centers), _p(sc.feats), _p(sc.values), m._wtp, m._bp,
                                       _p(self.outl), _p(self.n_outl), self.outl_cap,
                                       _p(self.field), REFINE_ABOVE, _p(self.refine_rows),
                                       _p(self.n_refine), self.outl_cap, _p(self.err), s),
              "field_exact_dev")
        check(LIB.nsvf_field_refine_fp32_dev(_p(self.refine_rows), _p(self.n_refine),
                                             self.outl_cap, C, _p(self.n_hit), _p(self.offset),
                                             self.cap, _p(self.vox), _p(self.xyzd),
                                             sc.centers.size(0), sc.values.size(0), sc.voxel_size,
                                             _p(sc.centers), _p(sc.feats), _p(sc.values), m._wtp,
                                             m._bp, _p(self.field), s), "field_refine_fp32_dev")
        self.colors.copy_(self.bg.expand(C, 3))
        self.depths.fill_(sc.bg_depth)
        self.missed.fill_(1.0)
        check(LIB.nsvf_composite_segments_dev(C, _p(self.n_hit), _p(self.offset), self.cap,
                                              _p(self.field),
                                              _p(self.xyzd), _p(self.sdepth), _p(self.pix), 7.0,
                                              sc.bg, sc.bg_depth, _p(self.colors),
                                              _p(self.depths), _p(self.missed), 1, s),
              "composite_segments_dev")

    def capture(self):
        """Record the chain into a CUDA graph (one eager run first: it sets the
        kernels' attributes and lets torch's allocator settle)."""
        self.cam.copy_(torch.from_numpy(camera_params([0.0, 0.0, 4.0], 64, 64, 80.0)))
        with torch.cuda.stream(self.stream):
            self._enqueue()
        self.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self._enqueue()
        self.stream.synchronize()
        self.err.zero_()
        self.graph = g

    def launch(self, cam18):
        """Render the chunk described by `cam18`, asynchronously on self.stream."""
        self.cam_host.copy_(torch.from_numpy(cam18))
        with torch.cuda.stream(self.stream):
            self.cam.copy_(self.cam_host, non_blocking=True)
            if self.use_graph and self.graph is not None:
                self.graph.replay()
            else:
                self._enqueue()


class SceneStore:
    """Resident scenes, with their bytes (octree, corner table, embeddings,
    MLP weights) counted against an HBM budget."""

    def __init__(self, device, hbm_budget_bytes):
        self.device = device
        self.budget = int(hbm_budget_bytes)
        self.scenes = {}
        self.used = 0

    def add(self, scene_id, encoder, field):
        st = SceneState(encoder, field)
        b = st.bytes()
        if self.used + b > self.budget:
            raise MemoryError("scene %r (%d bytes) exceeds the HBM budget" % (scene_id, b))
        self.scenes[scene_id] = st
        self.used += b
        return st


class Request:
    def __init__(self, rid, scene_id, cam, width, height, focal, arrival=0.0):
        self.rid, self.scene_id = rid, scene_id
        self.cam = np.asarray(cam, np.float64)
        self.width, self.height, self.focal = int(width), int(height), float(focal)
        self.arrival = float(arrival)
        self.rays = self.width * self.height
        self.next_chunk = 0
        self.done_chunks = 0
        self.n_chunks = 0
        self.colors = self.depths = None
        self.t_admit = self.t_done = None
        self.redo = []

    def latency(self):
        return self.t_done - self.arrival


class Server:
    """Continuous-batching request loop over ChunkPipeline slots.

    `frame_budget_bytes` bounds the host+device bytes of admitted frames
    (outputs: 16 B per pixel); `max_inflight` bounds admitted frames;
    `slots` is the number of chunks on the GPU at once (one stream each).
    Each (slot, scene) pair keeps a captured pipeline of `chunk_rays` rays
    holding up to `chunk_rays * samples_per_ray` samples (40 B each, plus
    28 B x max_hits per ray of hit lists): about 1.8 GB per pipeline at the
    defaults. On the 8-scene serving workload 256k-ray chunks gave the best
    capacity and tail latency (64k: 99 M rays/s, p99 20 ms; 256k: 126 M,
    p99 10 ms)."""

    def __init__(self, store, chunk_rays=262144, slots=3, max_inflight=8,
                 frame_budget_bytes=1 << 30, samples_per_ray=128, use_graph=True):
        self.store = store
        self.C = int(chunk_rays)
        self.max_inflight = max_inflight
        self.frame_budget = frame_budget_bytes
        self.device = store.device
        self.streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self.pipes = {}
        self.samples_per_ray = samples_per_ray
        self.use_graph = use_graph
        self.pool = []          # pinned host frame buffers, reused across requests

    def _host_buffers(self, rays):
        for i, (c, d, e) in enumerate(self.pool):
            if c.shape[0] >= rays:
                self.pool.pop(i)
                return c, d, e
        n_chunks = max(1, math.ceil(rays / self.C))
        return (torch.empty(rays, 3, dtype=torch.float32).pin_memory(),
                torch.empty(rays, dtype=torch.float32).pin_memory(),
                torch.zeros(n_chunks, dtype=torch.int32).pin_memory())

    def reserve_host_buffers(self, rays, n):
        """Pin n frame buffers of `rays` pixels ahead of serving."""
        for _ in range(n):
            self.pool.append(self._host_buffers(rays))
        self.pool.sort(key=lambda b: b[0].shape[0])

    def pipe(self, slot, scene_id):
        key = (slot, scene_id)
        p = self.pipes.get(key)
        if p is None:
            p = ChunkPipeline(self.store.scenes[scene_id], self.C, self.samples_per_ray,
                              self.streams[slot], self.use_graph)
            if self.use_graph:
                p.capture()
            self.pipes[key] = p
        return p

    def warm(self, scene_ids):
        """Build (and capture) every slot's pipeline for these scenes up front."""
        for sid in scene_ids:
            for s in range(len(self.streams)):
                self.pipe(s, sid)
        torch.cuda.synchronize(self.device)

    def _frame_bytes(self, r):
        return r.rays * 16

    def run(self, requests, real_time=True):
        """Serve `requests` (arrival times in seconds from the start). With
        real_time the arrivals follow the wall clock; otherwise every request
        is present from the start. Returns the requests with colors/depths
        (host tensors) and latencies filled in."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = time.perf_counter()
        arriving = deque(reqs)
        waiting = deque()
        inflight = []
        busy = [None] * len(self.streams)
        done = 0
        used = 0
        while done < len(reqs):
            now = time.perf_counter() - t0
            while arriving and (not real_time or arriving[0].arrival <= now):
                waiting.append(arriving.popleft())
            # admission: slots and frame-buffer memory
            while waiting and len(inflight) < self.max_inflight and \
                    used + self._frame_bytes(waiting[0]) <= self.frame_budget:
                r = waiting.popleft()
                r.n_chunks = math.ceil(r.rays / self.C)
                r._bufs = self._host_buffers(r.rays)
                r.colors, r.depths, r.err = r._bufs[0][:r.rays], r._bufs[1][:r.rays], r._bufs[2]
                if r.err.shape[0] < r.n_chunks:
                    r.err = torch.zeros(r.n_chunks, dtype=torch.int32).pin_memory()
                r.t_admit = time.perf_counter() - t0
                used += self._frame_bytes(r)
                inflight.append(r)
            progressed = False
            # retire finished chunks
            for s, b in enumerate(busy):
                if b is not None and b[1].query():
                    r, _, k = b
                    busy[s] = None
                    progressed = True
                    r.done_chunks += 1
                    if int(r.err[k]) & (2 | 16):
                        r.redo.append(k)
                    if r.done_chunks == r.n_chunks:
                        for kk in r.redo:
                            self._redo_chunk(r, kk)
                        r.t_done = time.perf_counter() - t0
                        r.colors = r.colors.clone()
                        r.depths = r.depths.clone()
                        self.pool.append(r._bufs)
                        self.pool.sort(key=lambda b: b[0].shape[0])
                        del r._bufs
                        used -= self._frame_bytes(r)
                        inflight.remove(r)
                        done += 1
            # give every free slot the next chunk of the oldest frame
            for s in range(len(busy)):
                if busy[s] is not None:
                    continue
                r = next((x for x in inflight if x.next_chunk < x.n_chunks), None)
                if r is None:
                    break
                k = r.next_chunk
                r.next_chunk += 1
                first = k * self.C
                count = min(self.C, r.rays - first)
                p = self.pipe(s, r.scene_id)
                p.launch(camera_params(r.cam, r.width, r.height, r.focal, first, count))
                with torch.cuda.stream(p.stream):
                    r.colors[first:first + count].copy_(p.colors[:count], non_blocking=True)
                    r.depths[first:first + count].copy_(p.depths[:count], non_blocking=True)
                    r.err[k:k + 1].copy_(p.err, non_blocking=True)
                    p.err.zero_()
                    ev = torch.cuda.Event()
                    ev.record(p.stream)
                busy[s] = (r, ev, k)
                progressed = True
            if not progressed:
                time.sleep(0.0002)
        return reqs

    def _redo_chunk(self, r, k):
        """A chunk that overflowed its pipeline's sample capacity, rendered
        again with the synchronising served path."""
        sc = self.store.scenes[r.scene_id]
        first = k * self.C
        count = min(self.C, r.rays - first)
        cam = torch.from_numpy(camera_params(r.cam, r.width, r.height, r.focal, first, count)).to(self.device)
        ro = torch.empty(count, 3, device=self.device)
        rd = torch.empty(count, 3, device=self.device)
        check(LIB.nsvf_pinhole_rays(count, _p(cam), _p(ro), _p(rd),
                                    torch.cuda.current_stream(self.device).cuda_stream), "pinhole_rays")
        out = render_frame(sc, ro, rd)
        r.colors[first:first + count].copy_(out["colors"].cpu())
        r.depths[first:first + count].copy_(out["depths"].cpu())


def poisson_requests(n, rate, scene_ids, resolutions, seed=0, radius=4.0):
    """n requests with exponential inter-arrival times (mean 1/rate), a
    uniform scene and resolution each, and a seeded camera on the sphere."""
    rng = np.random.RandomState(seed)
    t = 0.0
    out = []
    cams = scenes.sphere_cameras(n, radius, seed + 1)
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        res = resolutions[rng.randint(len(resolutions))]
        sid = scene_ids[rng.randint(len(scene_ids))]
        out.append(Request(i, sid, cams[i], res, res, 80.0 * res / 64.0, t))
    return out
