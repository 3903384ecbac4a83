"""Multi-scene serving: continuous batching of ray chunks under CUDA graphs.

Frames are cut into pieces of PIECE_PIXELS consecutive pixels (the last one
shorter). A chunk is up to MAX_PIECES pieces of one scene's frames -- of the
oldest frame first, then of the next admitted frames of the same scene, of
any resolution -- so that small frames (a 128x128 frame is one piece) share
launches with each other and with the tails of large ones.

* ``ChunkPipeline`` renders one chunk of one scene with the served chain, from
  fixed device buffers and with no host synchronisation:
  1. pinhole rays of every piece from a table of camera parameters in device
     memory (`nsvf_pinhole_rays_multi`);
  2. SVO intersection in depth order (`nsvf_svo_intersect_grid`, the leaf-grid sweep;
     `nsvf_svo_intersect_sorted` for trees not in leaf-grid form);
  3. order-preserving hit compaction (torch cumsum + `nsvf_compact_hits`) and
     each piece's hit-row range (`nsvf_piece_rows`);
  4. the hit rays' lists and sampling distribution (`nsvf_gather_probs`);
  5. inverse-CDF sample count, offsets and compaction in one pass with a
     launch layout of its own per piece (`nsvf_sample_scan_compact_pieces`;
     `nsvf_sample_count_pieces` + `nsvf_sample_compact_pieces` for more than
     128 hit slots), so a piece renders the same whatever else
     shares its chunk;
  6. interpolation + tcgen05 BF16 MLP on the device-side sample count (`nsvf_field_samples_bf16_dev`),
     then the double-float re-evaluation of the samples far outside their voxel (`nsvf_field_exact_dev`)
     and the FP32 re-evaluation of the rays where such a sample's colour is large
     (`nsvf_field_refine_fp32_dev`);
  7. compensated compositing + background into the chunk's output (`nsvf_composite_segments_dev`).

  It is captured once into a CUDA graph and replayed per chunk. The only
  per-chunk input is the camera table (18 floats per piece, its first pixel
  and pixel count included) and the piece count, copied into the pipeline's
  parameter buffers before the replay.
* ``SceneStore`` holds resident scenes (`SceneState`), counted against an HBM
  budget.
* ``Server`` is the request loop:
  - A request (scene, camera, resolution) is admitted when an in-flight slot
    and enough of the host frame-buffer budget are free.
  - Every free pipeline slot takes the next chunk: pieces of the oldest
    admitted frame with pieces left, then of the other admitted frames of
    that scene. Chunks of different scenes run on the GPU at the same time,
    on separate streams.
  - Pipelines (one per slot and scene, created when first needed) are
    counted against the same HBM budget as the scenes: when a new one does
    not fit, the least recently used idle pipelines are released; if none
    is idle, the chunk waits for a slot to finish.
  - A frame completes when all its pieces are composited and copied to its
    pinned host buffer. Its latency is completion minus arrival.

A pipeline holds at most `chunk_rays * samples_per_ray` samples. A chunk that
needs more sets bit 1 of its error word (bit 4 for more far-outside samples
than its list holds); the server then renders each of its pieces again with
the synchronising served path (`render_frame`, whose launch layout for a piece
alone is the piece's own), so results never depend on the capacity.
"""
import math
import time
from collections import OrderedDict, deque

import numpy as np
import torch

from . import scenes
from ._lib import LIB, check
from .served import REFINE_ABOVE, SceneState, render_frame

PIECE_PIXELS = 16384
MAX_PIECES = 16


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
    """Fixed-size, synchronisation-free render of one chunk (up to MAX_PIECES
    pixel ranges) of one scene."""

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

        self.cams = z(MAX_PIECES, 18)
        self.n_seg = z(1, dtype=i32)
        self.cams_host = torch.zeros(MAX_PIECES, 18, dtype=f32).pin_memory()
        self.n_seg_host = torch.zeros(1, dtype=i32).pin_memory()
        self.piece_rows = z(MAX_PIECES + 1, dtype=i64)
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
        # samples far outside their voxel, re-evaluated in double-float, and
        # the rays re-evaluated in FP32 (their such sample's colour is large)
        self.outl_cap = max(4096, self.cap // 1024)
        self.outl = z(self.outl_cap, dtype=i64)
        self.n_outl = z(1, dtype=i64)
        self.refine_rows = z(self.outl_cap, dtype=i64)
        self.n_refine = z(1, dtype=i64)
        self.ws = torch.empty(self._ws_bytes(scene, C), dtype=u8, device=dev)
        self.scan_ws = torch.empty(int(LIB.nsvf_sample_scan_bytes(C)), dtype=u8, device=dev)
        self.bg = torch.tensor(list(scene.bg), device=dev)
        self.graph = None
        self.use_graph = use_graph

    @staticmethod
    def estimate_bytes(scene, chunk_rays, samples_per_ray):
        """Device bytes of a pipeline, before it is created."""
        C, H = int(chunk_rays), scene.max_hits
        cap = C * int(samples_per_ray)
        outl = max(4096, cap // 1024)
        per_ray = 24 + 12 * H + 1 + 4 + 8 + 16 * H + 4 + 4 + 8 + 20
        return C * per_ray + cap * 40 + outl * 16 + ChunkPipeline._ws_bytes(scene, C) + \
            int(LIB.nsvf_sample_scan_bytes(C)) + MAX_PIECES * 80 + 64

    @staticmethod
    def _ws_bytes(scene, C):
        """Traversal scratch: the leaf-grid sweep's ray list (the scene holds
        the grid and its packed octree), else the depth-first kernel's packed
        octree."""
        if scene.svo_grid.ok:
            return max(16, int(LIB.nsvf_svo_grid_list_bytes(C)))
        return max(16, int(LIB.nsvf_svo_workspace_bytes(1, scene.octree_centers.shape[0])))

    def bytes(self):
        ts = [v for v in vars(self).values() if isinstance(v, torch.Tensor) and v.is_cuda]
        return sum(t.numel() * t.element_size() for t in ts)

    def _enqueue(self):
        sc, C, H, s = self.scene, self.C, self.scene.max_hits, self.stream.cuda_stream
        check(LIB.nsvf_pinhole_rays_multi(C, MAX_PIECES, _p(self.n_seg), _p(self.cams), _p(self.ro),
                                          _p(self.rd), s), "pinhole_rays_multi")
        if sc.svo_grid.ok:
            sc.svo_grid.intersect_into(C, H, _p(self.ro), _p(self.rd), _p(self.idx), _p(self.lo),
                                       _p(self.hi), _p(self.hits), s, list_ws=self.ws,
                                       err=self.err, padded=False)
        else:
            check(LIB.nsvf_svo_intersect_sorted(1, 1, sc.octree_centers.shape[0], C,
                                                sc.voxel_size, H, _p(self.ro), _p(self.rd),
                                                _p(sc.octree_centers), _p(sc.octree_children),
                                                _p(self.idx), _p(self.lo), _p(self.hi),
                                                _p(self.hits), _p(self.err), _p(self.ws), s),
                  "svo_intersect_sorted")
        torch.cumsum(self.hits, 0, dtype=torch.int32, out=self.scan)
        check(LIB.nsvf_compact_hits(C, _p(self.hits), _p(self.scan), _p(self.pix), _p(self.n_hit),
                                    s), "compact_hits")
        check(LIB.nsvf_piece_rows(MAX_PIECES, _p(self.n_seg), _p(self.cams), C, _p(self.scan),
                                  _p(self.piece_rows), s), "piece_rows")
        check(LIB.nsvf_gather_probs(C, _p(self.n_hit), H, sc.step_size, _p(self.pix), _p(self.idx),
                                    _p(self.lo), _p(self.hi), _p(self.I), _p(self.L), _p(self.U),
                                    _p(self.probs), _p(self.steps), s), "gather_probs")
        if H <= 128:
            check(LIB.nsvf_sample_scan_compact_pieces(
                C, _p(self.n_hit), H, _p(self.I), _p(self.L), _p(self.U), _p(self.probs),
                _p(self.steps), _p(self.piece_rows), MAX_PIECES, _p(self.ro), 3, _p(self.rd),
                _p(self.pix), _p(self.offset), self.cap, _p(self.vox), _p(self.xyzd),
                _p(self.sdepth), _p(self.scan_ws), self.scan_ws.numel(), _p(self.err), s),
                "sample_scan_compact_pieces")
        else:
            check(LIB.nsvf_sample_count_pieces(C, _p(self.n_hit), H, _p(self.I), _p(self.L),
                                               _p(self.U), _p(self.probs), _p(self.steps),
                                               _p(self.piece_rows), MAX_PIECES, _p(self.count), s),
                  "sample_count_pieces")
            torch.cumsum(self.count, 0, out=self.offset[1:])
            check(LIB.nsvf_sample_compact_pieces(C, _p(self.n_hit), H, _p(self.I), _p(self.L),
                                                 _p(self.U), _p(self.probs), _p(self.steps),
                                                 _p(self.piece_rows), MAX_PIECES, _p(self.ro), 3,
                                                 _p(self.rd), _p(self.pix), _p(self.offset),
                                                 self.cap, _p(self.vox), _p(self.xyzd),
                                                 _p(self.sdepth), _p(self.err), s),
                  "sample_compact_pieces")
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
        self.cams.zero_()
        self.cams[0].copy_(torch.from_numpy(camera_params([0.0, 0.0, 4.0], 64, 64, 80.0)))
        self.n_seg.fill_(1)
        with torch.cuda.stream(self.stream):
            self._enqueue()
        self.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self._enqueue()
        self.stream.synchronize()
        self.err.zero_()
        self.graph = g

    def launch(self, cams):
        """Render the chunk whose pieces are the camera rows `cams` [n, 18]
        (n <= MAX_PIECES; their counts sum to at most chunk_rays),
        asynchronously on self.stream. The host-side tables are reused, so
        the previous launch on this pipeline must have been retired."""
        n = len(cams)
        self.cams_host.zero_()
        self.cams_host[:n].copy_(torch.from_numpy(np.stack(cams)))
        self.n_seg_host.fill_(n)
        with torch.cuda.stream(self.stream):
            self.cams.copy_(self.cams_host, non_blocking=True)
            self.n_seg.copy_(self.n_seg_host, non_blocking=True)
            if self.use_graph and self.graph is not None:
                self.graph.replay()
            else:
                self._enqueue()


class SceneStore:
    """Resident scenes, with their bytes (octree, corner table, embeddings,
    MLP weights) counted against an HBM budget. The serving pipelines are
    counted against the same budget by the Server."""

    def __init__(self, device, hbm_budget_bytes):
        self.device = device
        self.budget = int(hbm_budget_bytes)
        self.scenes = {}
        self.used = 0

    def add(self, scene_id, encoder, field):
        """Make a scene resident. The scene's data is the caller's, so a scene
        that does not fit is refused (MemoryError) rather than evicting
        another; remove() one first."""
        st = SceneState(encoder, field)
        b = st.bytes()
        if self.used + b > self.budget:
            raise MemoryError("scene %r (%d bytes) exceeds the HBM budget" % (scene_id, b))
        self.scenes[scene_id] = st
        self.used += b
        return st

    def remove(self, scene_id):
        st = self.scenes.pop(scene_id)
        self.used -= st.bytes()


class Request:
    def __init__(self, rid, scene_id, cam, width, height, focal, arrival=0.0):
        self.rid, self.scene_id = rid, scene_id
        self.cam = np.asarray(cam, np.float64)
        self.width, self.height, self.focal = int(width), int(height), float(focal)
        self.arrival = float(arrival)
        self.rays = self.width * self.height
        self.pieces = [(f, min(PIECE_PIXELS, self.rays - f)) for f in range(0, self.rays, PIECE_PIXELS)]
        self.next_piece = 0
        self.done_pieces = 0
        self.colors = self.depths = None
        self.t_admit = self.t_done = None
        self.redo = []

    def latency(self):
        return self.t_done - self.arrival


class Server:
    """Continuous-batching request loop over ChunkPipeline slots.

    `frame_budget_bytes` bounds the pinned host bytes of admitted frames
    (16 B per pixel); `max_inflight` bounds admitted frames; `slots` is the
    number of chunks on the GPU at once (one stream each). Each (slot,
    scene) pair gets a captured pipeline of `chunk_rays` rays holding up to
    `chunk_rays * samples_per_ray` samples (40 B each, plus 28 B x max_hits
    per ray of hit lists: about 1.8 GB at the defaults), counted with the
    scenes against the store's HBM budget (`hbm_budget_bytes` overrides it);
    idle pipelines are released, least recently used first, to make room.
    On the 8-scene serving workload 256k-ray chunks gave the best capacity
    and tail latency."""

    def __init__(self, store, chunk_rays=262144, slots=3, max_inflight=8,
                 frame_budget_bytes=1 << 30, samples_per_ray=128, use_graph=True,
                 hbm_budget_bytes=None):
        if chunk_rays % PIECE_PIXELS:
            raise ValueError("chunk_rays must be a multiple of %d" % PIECE_PIXELS)
        self.store = store
        self.C = int(chunk_rays)
        self.max_inflight = max_inflight
        self.frame_budget = frame_budget_bytes
        self.hbm_budget = int(hbm_budget_bytes) if hbm_budget_bytes is not None else store.budget
        self.device = store.device
        self.streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self.pipes = OrderedDict()      # (slot, scene) -> pipeline, least recently used first
        self.pipe_bytes = 0
        self.samples_per_ray = samples_per_ray
        self.use_graph = use_graph
        self.pool = []          # pinned host frame buffers, reused across requests
        self.err_host = [torch.zeros(1, dtype=torch.int32).pin_memory() for _ in range(slots)]
        self.stats = {"chunks": 0, "pieces": 0, "max_frames_per_chunk": 0, "pipelines_released": 0}

    def _host_buffers(self, rays):
        for i, (c, d) in enumerate(self.pool):
            if c.shape[0] >= rays:
                self.pool.pop(i)
                return c, d
        return (torch.empty(rays, 3, dtype=torch.float32).pin_memory(),
                torch.empty(rays, dtype=torch.float32).pin_memory())

    def reserve_host_buffers(self, rays, n):
        """Pin n frame buffers of `rays` pixels ahead of serving."""
        for _ in range(n):
            self.pool.append(self._host_buffers(rays))
        self.pool.sort(key=lambda b: b[0].shape[0])

    def device_bytes(self):
        return self.store.used + self.pipe_bytes

    def pipe(self, slot, scene_id, busy_keys=()):
        """The (slot, scene) pipeline, created (and captured) if needed once
        the HBM budget has room, releasing idle pipelines if it has not. None
        if nothing can be released now."""
        key = (slot, scene_id)
        p = self.pipes.get(key)
        if p is not None:
            self.pipes.move_to_end(key)
            return p
        sc = self.store.scenes[scene_id]
        need = ChunkPipeline.estimate_bytes(sc, self.C, self.samples_per_ray)
        while self.device_bytes() + need > self.hbm_budget:
            victim = next((k for k in self.pipes if k not in busy_keys), None)
            if victim is None:
                return None
            old = self.pipes.pop(victim)
            self.pipe_bytes -= old.bytes()
            old.stream.synchronize()
            del old
            self.stats["pipelines_released"] += 1
        p = ChunkPipeline(sc, self.C, self.samples_per_ray, self.streams[slot], self.use_graph)
        if self.use_graph:
            p.capture()
        self.pipes[key] = p
        self.pipe_bytes += p.bytes()
        return p

    def warm(self, scene_ids):
        """Build (and capture) every slot's pipeline for these scenes up front
        (as far as the HBM budget allows)."""
        for sid in scene_ids:
            for s in range(len(self.streams)):
                self.pipe(s, sid)
        torch.cuda.synchronize(self.device)

    def _frame_bytes(self, r):
        return r.rays * 16

    def _next_chunk(self, inflight):
        """Pieces for one chunk: the oldest frame with pieces left, then the
        other admitted frames of its scene, in arrival order, until the chunk
        is full. Returns (scene_id, [(request, piece index, chunk offset)])."""
        first = next((r for r in inflight if r.next_piece < len(r.pieces)), None)
        if first is None:
            return None, []
        sid = first.scene_id
        out, used = [], 0
        for r in inflight:
            if r.scene_id != sid:
                continue
            while r.next_piece < len(r.pieces) and len(out) < MAX_PIECES:
                k = r.next_piece
                cnt = r.pieces[k][1]
                if used + cnt > self.C:
                    break
                out.append((r, k, used))
                used += cnt
                r.next_piece += 1
            if len(out) >= MAX_PIECES or used >= self.C:
                break
        return sid, out

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
            # admission: in-flight slots and host frame-buffer memory
            while waiting and len(inflight) < self.max_inflight and \
                    used + self._frame_bytes(waiting[0]) <= self.frame_budget:
                r = waiting.popleft()
                r._bufs = self._host_buffers(r.rays)
                r.colors, r.depths = r._bufs[0][:r.rays], r._bufs[1][:r.rays]
                r.t_admit = time.perf_counter() - t0
                used += self._frame_bytes(r)
                inflight.append(r)
            progressed = False
            # retire finished chunks
            for s, b in enumerate(busy):
                if b is None or not b[1].query():
                    continue
                chunk, _, _ = b
                busy[s] = None
                progressed = True
                bad = int(self.err_host[s][0]) & (2 | 16)
                for r, k, _ in chunk:
                    r.done_pieces += 1
                    if bad:
                        r.redo.append(k)
                    if r.done_pieces == len(r.pieces):
                        for kk in r.redo:
                            self._redo_piece(r, kk)
                        r.t_done = time.perf_counter() - t0
                        r.colors = r.colors.clone()
                        r.depths = r.depths.clone()
                        self.pool.append(r._bufs)
                        self.pool.sort(key=lambda b: b[0].shape[0])
                        del r._bufs
                        used -= self._frame_bytes(r)
                        inflight.remove(r)
                        done += 1
            # give every free slot the next chunk
            busy_keys = {b[2] for b in busy if b is not None}
            for s in range(len(busy)):
                if busy[s] is not None:
                    continue
                sid = next((r.scene_id for r in inflight if r.next_piece < len(r.pieces)), None)
                if sid is None:
                    break
                p = self.pipe(s, sid, busy_keys)
                if p is None:
                    continue          # no room for a pipeline now: wait for a slot
                sid, chunk = self._next_chunk(inflight)
                cams = [camera_params(r.cam, r.width, r.height, r.focal, *r.pieces[k])
                        for r, k, _ in chunk]
                p.launch(cams)
                with torch.cuda.stream(p.stream):
                    for r, k, off in chunk:
                        first, cnt = r.pieces[k]
                        r.colors[first:first + cnt].copy_(p.colors[off:off + cnt], non_blocking=True)
                        r.depths[first:first + cnt].copy_(p.depths[off:off + cnt], non_blocking=True)
                    self.err_host[s].copy_(p.err, non_blocking=True)
                    p.err.zero_()
                    ev = torch.cuda.Event()
                    ev.record(p.stream)
                busy[s] = (chunk, ev, (s, sid))
                busy_keys.add((s, sid))
                self.stats["chunks"] += 1
                self.stats["pieces"] += len(chunk)
                self.stats["max_frames_per_chunk"] = max(self.stats["max_frames_per_chunk"],
                                                         len({r.rid for r, _, _ in chunk}))
                progressed = True
            if not progressed:
                time.sleep(0.0002)
        return reqs

    def _redo_piece(self, r, k):
        """A piece whose chunk overflowed its pipeline's capacity, rendered
        again alone with the synchronising served path."""
        sc = self.store.scenes[r.scene_id]
        first, count = r.pieces[k]
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
