"""Loader of the C-ABI library (nsvf_gb300/_build/libnsvf_gb300.so).

The library is the product: there is no CPU or PyTorch fallback. If it is
missing, importing this module raises, naming the build command.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# NSVF_GB300_LIB names a library built elsewhere (same sources, another
# output directory); by default the in-tree build is loaded.
LIB_PATH = os.environ.get("NSVF_GB300_LIB") or os.path.join(HERE, "_build", "libnsvf_gb300.so")

NSVF_OK = 0


class NsvfError(RuntimeError):
    pass


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "nsvf_gb300: %s is missing; build it with `python -m nsvf_gb300.build` "
            "(or __graft_entry__.build())" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
    sig = {
        "nsvf_status_string": ([i32], ctypes.c_char_p),
        "nsvf_launch_count": ([], ctypes.c_longlong),
        "nsvf_aabb_intersect": ([i32, i32, i32, i32, f32, i32, P, P, P, P, P, P, P], i32),
        "nsvf_svo_workspace_bytes": ([i32, i32], i64),
        "nsvf_svo_intersect": ([i32, i32, i32, i32, f32, i32, P, P, P, P, P, P, P, P, P, P], i32),
        "nsvf_svo_intersect_sorted": ([i32, i32, i32, i32, f32, i32, P, P, P, P, P, P, P, P, P,
                                       P, P], i32),
        "nsvf_svo_pack": ([i32, f32, P, P, P, P], i32),
        "nsvf_svo_grid_build": ([i32, f32, P, P, P, i64, P], i32),
        "nsvf_svo_grid_info": ([P, P], i32),
        "nsvf_svo_grid_list_bytes": ([i64], i64),
        "nsvf_svo_intersect_grid": ([i64, i32, f32, i32, P, P, P, P, P, P, P, P, P, P, P, P, P,
                                     P], i32),
        "nsvf_svo_intersect_grid_rows": ([i64, i32, f32, i32, P, P, P, P, P, P, P, P, P, P, P, P,
                                          P, i32, P], i32),
        "nsvf_ball_intersect": ([i32, i32, i32, i32, f32, i32, P, P, P, P, P, P, P], i32),
        "nsvf_triangle_intersect": ([i32, i32, i32, i32, f32, f32, i32, P, P, P, P, P, P, P], i32),
        "nsvf_uniform_ray_sampling": ([i32, i32, i32, i32, f32, P, P, P, P, P, P, P, P, P], i32),
        "nsvf_inverse_cdf_sampling": ([i64, i32, i32, i32, f32, P, P, P, P, P, P, P, P, P, P,
                                       P, P, P], i32),
        "nsvf_build_octree": ([P, P, i64, i32, P, P, i64], i64),
        "nsvf_trilinear_embed": ([i64, i32, f32, i64, i64, P, i32, P, P, P, i32, P, P, P, P], i32),
        "nsvf_trilinear_embed_backward": ([i64, i32, f32, i64, i64, P, i32, P, P, P, i32, P, P, P,
                                           P, P], i32),
        "nsvf_composite": ([i64, i32, P, P, P, P, P, P, P, i32, P], i32),
        "nsvf_composite_backward": ([i64, i32, P, P, P, P, P, P, P, P, P, i32, P], i32),
        "nsvf_mlp_forward_bf16": ([i64, P, P, P, P, P, P], i32),
        "nsvf_field_samples_bf16": ([i64, P, P, i64, i64, f32, P, P, P, P, P, P, P, P], i32),
        "nsvf_prune_scores_bf16": ([i64, i32, i32, f32, i64, f32, P, P, P, P, P, P, P, P], i32),
        "nsvf_sample_count": ([i64, i32, P, P, P, P, P, P, P, P], i32),
        "nsvf_sample_compact": ([i64, i32, P, P, P, P, P, P, P, i64, P, P, P, P, P, P, P], i32),
        "nsvf_composite_segments": ([i64, P, P, P, P, P, f32, P, f32, P, P, P, i32, P], i32),
        "nsvf_pinhole_rays": ([i64, P, P, P, P], i32),
        "nsvf_camera_rays": ([i64, P, P, P, P], i32),
        "nsvf_compact_hits": ([i64, P, P, P, P, P], i32),
        "nsvf_gather_probs": ([i64, P, i32, f32, P, P, P, P, P, P, P, P, P, P], i32),
        "nsvf_ray_probs": ([i64, i32, f32, P, P, P, P, P, P], i32),
        "nsvf_pinhole_rays_multi": ([i64, i32, P, P, P, P, P], i32),
        "nsvf_piece_rows": ([i32, P, P, i64, P, P, P], i32),
        "nsvf_sample_count_pieces": ([i64, P, i32, P, P, P, P, P, P, i32, P, P], i32),
        "nsvf_sample_compact_pieces": ([i64, P, i32, P, P, P, P, P, P, i32, P, i64, P, P, P, i64,
                                        P, P, P, P, P], i32),
        "nsvf_parallel_ray_sampling": ([i64, i32, i32, f32, P, P, P, P, i32, P, P, P, P, P], i32),
        "nsvf_parallel_sampling_smem_bytes": ([i32, i32], i64),
        "nsvf_prune_screen_bf16": ([i64, i32, i32, f32, f32, f32, i64, f32, P, P, P, P, P, P, P,
                                    P, P, i64, P, P], i32),
        "nsvf_prune_exact_dev": ([i64, i32, i32, ctypes.c_double, i64, f32, P, P, P, P, P, P, P,
                                  i64, P, P, P], i32),
        "nsvf_sample_count_dev": ([i64, P, i32, P, P, P, P, P, P, P], i32),
        "nsvf_sample_compact_dev": ([i64, P, i32, P, P, P, P, P, P, i64, P, P, P, i64, P, P, P,
                                     P, P], i32),
        "nsvf_sample_scan_bytes": ([i64], i64),
        "nsvf_sample_scan_compact_dev": ([i64, P, i32, P, P, P, P, P, P, i64, P, P, P, i64, P, P,
                                          P, P, i64, P, P], i32),
        "nsvf_sample_scan_compact_pieces": ([i64, P, i32, P, P, P, P, P, P, i32, P, i64, P, P, P,
                                             i64, P, P, P, P, i64, P, P], i32),
        "nsvf_composite_segments_dev": ([i64, P, P, i64, P, P, P, P, f32, P, f32, P, P, P, i32, P],
                                        i32),
        "nsvf_field_samples_bf16_dev": ([i64, P, P, P, i64, i64, f32, P, P, P, P, P, P, P, P, i64,
                                         P, P], i32),
        "nsvf_field_samples_fp8": ([i64, P, P, i64, i64, f32, P, P, P, P, P, P, P, P, P], i32),
        "nsvf_field_samples_fp8_dev": ([i64, P, P, P, i64, i64, f32, P, P, P, P, P, P, P, P, P,
                                        i64, P, P], i32),
        "nsvf_flag_outliers": ([i64, P, P, P, i64, f32, P, P, P, i64, P, P], i32),
        "nsvf_field_exact_dev": ([i64, P, P, P, P, i64, P, P, P, i64, i64, f32, P, P, P, P, P, P,
                                  P, i64, P, f32, P, P, i64, P, P], i32),
        "nsvf_field_refine_fp32_dev": ([P, P, i64, i64, P, P, i64, P, P, i64, i64, f32, P, P, P, P,
                                        P, P, P], i32),
        "nsvf_wait_timeout_selftest": ([ctypes.c_uint64, P, P], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


LIB = _load()


def check(status, what):
    if status != NSVF_OK:
        msg = LIB.nsvf_status_string(int(status)).decode()
        raise NsvfError("nsvf_gb300: %s failed: %s (%d)" % (what, msg, status))
    return status


def exported_symbols():
    """Names declared in include/nsvf_gb300.h that the library must export."""
    return [
        "nsvf_status_string", "nsvf_launch_count", "nsvf_aabb_intersect", "nsvf_svo_workspace_bytes",
        "nsvf_svo_intersect", "nsvf_svo_intersect_sorted", "nsvf_svo_pack",
        "nsvf_svo_grid_build", "nsvf_svo_grid_info", "nsvf_svo_grid_list_bytes",
        "nsvf_svo_intersect_grid", "nsvf_svo_intersect_grid_rows", "nsvf_ball_intersect",
        "nsvf_triangle_intersect",
        "nsvf_uniform_ray_sampling", "nsvf_inverse_cdf_sampling", "nsvf_build_octree",
        "nsvf_trilinear_embed", "nsvf_trilinear_embed_backward", "nsvf_composite",
        "nsvf_composite_backward", "nsvf_mlp_forward_bf16", "nsvf_sample_count",
        "nsvf_sample_compact", "nsvf_composite_segments", "nsvf_field_samples_bf16",
        "nsvf_prune_scores_bf16", "nsvf_pinhole_rays", "nsvf_camera_rays", "nsvf_compact_hits",
        "nsvf_gather_probs", "nsvf_sample_count_dev", "nsvf_sample_compact_dev", "nsvf_composite_segments_dev",
        "nsvf_field_samples_bf16_dev", "nsvf_field_samples_fp8", "nsvf_field_samples_fp8_dev",
        "nsvf_wait_timeout_selftest", "nsvf_flag_outliers", "nsvf_field_exact_dev",
        "nsvf_ray_probs", "nsvf_prune_screen_bf16", "nsvf_prune_exact_dev",
        "nsvf_field_refine_fp32_dev", "nsvf_parallel_ray_sampling",
        "nsvf_parallel_sampling_smem_bytes", "nsvf_pinhole_rays_multi", "nsvf_piece_rows",
        "nsvf_sample_count_pieces", "nsvf_sample_compact_pieces",
        "nsvf_sample_scan_bytes", "nsvf_sample_scan_compact_dev", "nsvf_sample_scan_compact_pieces",
    ]
