"""Import the reference's pure-PyTorch modules on the CPU.

TEST INFRASTRUCTURE ONLY, used where the reference checkout exists (this
container): tests/golden/make_golden.py runs the reference code through it to
produce the committed golden fixtures, and CPU tests compare the numpy oracle
against it.

The reference imports packages that are absent here (fairseq, plyfile, cv2,
imageio, skimage, pandas, pylab, torchvision, open3d). They are replaced by
empty modules; fairseq's LayerNorm becomes nn.LayerNorm. Modules are loaded
by file path in dependency order. fairnr/modules/reader.py is NOT loaded: it
turns on torch.autograd.set_detect_anomaly(True) for the whole process
(fairnr/modules/reader.py:12).

``fairnr.clib`` is loaded from the reference file, and its ``_ext`` (the CUDA
extension, which cannot be built here) is bound to ``CpuExt``, a stand-in
that runs the reference's own kernel bodies compiled for the CPU
(oracle.ref_clib) and its own octree builder (oracle/_ref/octree).
"""
import importlib.util
import os
import sys
import types

import numpy as np

from .build_ref import REF  # noqa: E402  (the reference checkout's location)
_STUBS = ["cv2", "pandas", "pylab", "skimage", "skimage.metrics", "imageio", "plyfile", "open3d",
          "fairseq", "fairseq.models", "fairseq.utils", "fairseq.modules", "fairseq.meters",
          "fairseq.distributed_utils", "fairseq.logging", "fairseq.logging.progress_bar",
          "fairseq.tasks", "fairseq.optim", "fairseq.optim.fp16_optimizer", "fairseq.data",
          "fairseq.criterions", "fairseq.metrics", "torchvision", "torchvision.utils"]
_mods = None


def available():
    return os.path.isdir(os.path.join(REF, "fairnr"))


class CpuExt:
    """Stand-in for fairnr.clib._ext backed by the reference code built for the CPU."""

    @staticmethod
    def _t(a):
        import torch
        return torch.from_numpy(np.ascontiguousarray(a))

    @classmethod
    def aabb_intersect(cls, ray_start, ray_dir, points, voxelsize, n_max):
        from oracle import ref_clib
        out = ref_clib.aabb_intersect(ray_start.numpy(), ray_dir.numpy(), points.numpy(),
                                      float(voxelsize), int(n_max))
        return tuple(cls._t(o) for o in out)

    @classmethod
    def svo_intersect(cls, ray_start, ray_dir, points, children, voxelsize, n_max):
        from oracle import ref_clib
        out = ref_clib.svo_intersect(ray_start.numpy(), ray_dir.numpy(), points.numpy(),
                                     children.numpy(), float(voxelsize), int(n_max))
        return tuple(cls._t(o) for o in out)

    @classmethod
    def uniform_ray_sampling(cls, pts_idx, min_depth, max_depth, noise, step_size, max_steps):
        from oracle import ref_clib
        out = ref_clib.uniform_ray_sampling(pts_idx.numpy(), min_depth.numpy(), max_depth.numpy(),
                                            noise.numpy(), float(step_size), int(max_steps))
        return tuple(cls._t(o) for o in out)

    @classmethod
    def inverse_cdf_sampling(cls, pts_idx, min_depth, max_depth, noise, probs, steps, fixed):
        from oracle import ref_clib
        out = ref_clib.inverse_cdf_sampling(pts_idx.numpy(), min_depth.numpy(), max_depth.numpy(),
                                            noise.numpy(), probs.numpy(), steps.numpy(), float(fixed))
        return tuple(cls._t(o) for o in out)

    @classmethod
    def ball_intersect(cls, ray_start, ray_dir, points, radius, n_max):
        from oracle import ref_clib
        out = ref_clib.ball_intersect(ray_start.numpy(), ray_dir.numpy(), points.numpy(),
                                      float(radius), int(n_max))
        return tuple(cls._t(o) for o in out)

    @classmethod
    def triangle_intersect(cls, ray_start, ray_dir, face_points, cagesize, blur, n_max):
        from oracle import ref_clib
        out = ref_clib.triangle_intersect(ray_start.numpy(), ray_dir.numpy(), face_points.numpy(),
                                          float(cagesize), float(blur), int(n_max))
        return tuple(cls._t(o) for o in out)

    @staticmethod
    def build_octree(center, points, depth):
        from oracle import build_ref
        return build_ref.build_octree().build_octree(center, points, depth)


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load():
    """Returns a namespace with the reference modules: clib, geometry,
    module_utils, implicit, field, renderer, encoder."""
    global _mods
    if _mods is not None:
        return _mods
    import torch.nn as nn
    for name in _STUBS:
        if name not in sys.modules:
            sys.modules[name] = types.ModuleType(name)
    m = sys.modules
    m["plyfile"].PlyData = m["plyfile"].PlyElement = object
    m["fairseq.modules"].LayerNorm = nn.LayerNorm
    m["fairseq.utils"].get_activation_fn = lambda x: None
    m["fairseq.meters"].StopwatchMeter = object
    for pkg in ["fairnr", "fairnr.data", "fairnr.modules"]:
        if pkg not in sys.modules:
            mm = types.ModuleType(pkg)
            mm.__path__ = []
            sys.modules[pkg] = mm
    R = os.path.join(REF, "fairnr")
    ext = types.ModuleType("fairnr.clib._ext")
    for name in ["aabb_intersect", "svo_intersect", "uniform_ray_sampling",
                 "inverse_cdf_sampling", "build_octree", "triangle_intersect", "ball_intersect"]:
        setattr(ext, name, getattr(CpuExt, name))
    sys.modules["fairnr.clib._ext"] = ext
    ns = types.SimpleNamespace()
    ns.clib = _load("fairnr.clib", os.path.join(R, "clib", "__init__.py"))
    ns.clib._ext = ext
    _load("fairnr.data.data_utils", os.path.join(R, "data", "data_utils.py"))
    ns.geometry = _load("fairnr.data.geometry", os.path.join(R, "data", "geometry.py"))
    ns.module_utils = _load("fairnr.modules.module_utils", os.path.join(R, "modules", "module_utils.py"))
    _load("fairnr.modules.hyper", os.path.join(R, "modules", "hyper.py"))
    ns.implicit = _load("fairnr.modules.implicit", os.path.join(R, "modules", "implicit.py"))
    ns.field = _load("fairnr.modules.field", os.path.join(R, "modules", "field.py"))
    ns.renderer = _load("fairnr.modules.renderer", os.path.join(R, "modules", "renderer.py"))
    ns.encoder = _load("fairnr.modules.encoder", os.path.join(R, "modules", "encoder.py"))
    _mods = ns
    return ns
