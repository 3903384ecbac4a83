"""Golden fixture of hierarchical resampling, from the reference itself (run
where the reference checkout is present):

    python tests/golden/make_golden_hier.py

On the 147-voxel scene of golden_small.npz: its deterministic coarse samples
and the coarse render's per-sample probabilities (render_probs) go through
the reference's prepare_hierarchical_sampling (fairnr/models/nerf.py:64-79,
and NSVFModel's override, fairnr/models/nsvf.py:83-87), then the reference
encoder's ray_sample places the fine samples (deterministic) and its
VolumeRenderer renders them with the same field. Two settings:

* nerf64 -- NeRFModel with fixed_fine_num_samples 64;
* nsvf2  -- NSVFModel with fine_num_sample_ratio 2 (steps = twice the
            coarse sample count of each ray).

The reference's model classes are loaded with fairseq stubbed (register
decorators as identities, BaseFairseqModel = nn.Module) and with a stub in
place of fairnr/modules/reader.py, which would switch autograd anomaly
detection on for the whole process. Writes golden_hier.npz: for each setting
the resampling inputs (min_depth, max_depth, intersected_voxel_idx, probs,
steps), the fine samples and the fine render's colors/depths/missed.
"""
import argparse
import contextlib
import importlib.util
import os
import sys
import types

import numpy as np
import torch
import torch.nn as nn

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import build_ref, ref_import  # noqa: E402
import make_golden as mg  # noqa: E402


def load_models(ref):
    m = sys.modules
    fm = m["fairseq.models"]
    fm.register_model = lambda name: (lambda cls: cls)
    fm.register_model_architecture = lambda a, b: (lambda f: f)
    fm.BaseFairseqModel = nn.Module

    @contextlib.contextmanager
    def with_torch_seed(seed):
        yield
    m["fairseq.utils"].with_torch_seed = with_torch_seed
    m["fairseq.utils"].item = lambda x: x
    reader = types.ModuleType("fairnr.modules.reader")
    reader.get_reader = lambda name: None
    m["fairnr.modules.reader"] = reader
    for pkg in ["fairnr.models"]:
        mm = types.ModuleType(pkg)
        mm.__path__ = []
        m[pkg] = mm
    R = os.path.join(ref_import.REF, "fairnr")

    def load(name, path):
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        m[name] = mod
        spec.loader.exec_module(mod)
        return mod
    load("fairnr.models.fairnr_model", os.path.join(R, "models", "fairnr_model.py"))
    nerf = load("fairnr.models.nerf", os.path.join(R, "models", "nerf.py"))
    nsvf = load("fairnr.models.nsvf", os.path.join(R, "models", "nsvf.py"))
    assert not torch.is_anomaly_enabled()
    return nerf.NeRFModel, nsvf.NSVFModel


def model_with_args(cls, **args):
    obj = cls.__new__(cls)
    nn.Module.__init__(obj)
    object.__setattr__(obj, "args", argparse.Namespace(**args))
    return obj


def main():
    ref = ref_import.load()
    build_ref.build_clib()
    NeRFModel, NSVFModel = load_models(ref)
    g = dict(np.load(os.path.join(HERE, "golden_small.npz")))
    pts, vs = g["points"], float(g["voxel_size"])
    embed = torch.from_numpy(g["embed"])
    weights = [(torch.from_numpy(g["W%d" % i]), torch.from_numpy(g["b%d" % i])) for i in range(5)]
    field = mg.StandInField(weights).eval()
    enc = mg.make_encoder(ref, pts, vs, True, embed)
    st = enc.precompute(id=None)
    hit = g["svo_hits"][0]
    rs = torch.from_numpy(g["ray_start"]).reshape(1, 3).expand(int(hit.sum()), 3)
    rd = torch.from_numpy(g["ray_dir"][hit])
    samples = {k: torch.from_numpy(g["svo_det_%s" % k]) for k in
               ["sampled_point_depth", "sampled_point_distance", "sampled_point_voxel_idx"]}
    all_results = {"probs": torch.from_numpy(g["render_probs"])}
    renderer = ref.renderer.VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    out = {}
    for tag, model in [("nerf64", model_with_args(NeRFModel, fixed_fine_num_samples=64)),
                       ("nsvf2", model_with_args(NSVFModel, fine_num_sample_ratio=2.0))]:
        io = model.prepare_hierarchical_sampling({}, dict(samples), all_results)
        for k in ["min_depth", "max_depth", "intersected_voxel_idx", "probs", "steps"]:
            out["%s_%s" % (tag, k)] = io[k].numpy()
        fine = enc.ray_sample(io)
        for k, v in fine.items():
            out["%s_fine_%s" % (tag, k)] = v.numpy()
        with torch.no_grad():
            res = renderer(enc, field.forward, rs, rd, dict(fine), st)
        for k in ["colors", "depths", "missed"]:
            out["%s_render_%s" % (tag, k)] = res[k].numpy()
    np.savez_compressed(os.path.join(HERE, "golden_hier.npz"), **out)
    print("wrote golden_hier.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
