"""ctypes declarations of include/millionsball.h.

Loading fails loudly: there is no CPU fallback anywhere in the package.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libmillionsball.so"

u8, u32, i64, f32 = C.c_uint8, C.c_uint32, C.c_int64, C.c_float
vp = C.c_void_p


class MbSettings(C.Structure):
    """struct mb_settings — PhysicsPlugin's fields (src/physics/mod.rs:53-85)."""

    _fields_ = [
        ("max_number_of_agents", u32),
        ("number_of_grids_one_dimension", u32),
        ("grid_size", u32),
        ("half_map_height", u32),
        ("gravity", f32 * 3),
        ("e_envir", f32),
        ("e_agent", f32),
        ("k_agent", f32),
        ("c_agent", f32),
        ("r_agent", f32),
        ("time_delta", f32),
        ("enable_simulation", u8),
        ("enable_spring", u8),
        ("exact_constants", u8),
        ("reserved0", u8),
    ]


class MbConsts(C.Structure):
    """struct mb_consts — the quantised constants the kernels run with."""

    _fields_ = [
        ("number_of_grids_one_dimension", u32),
        ("grid_size", u32),
        ("half_map_height", f32),
        ("half_map_size", f32),
        ("gravity", f32 * 3),
        ("e_envir", f32),
        ("e_agent", f32),
        ("k_agent", f32),
        ("c_agent", f32),
        ("r_agent", f32),
        ("time_delta", f32),
        ("enable_spring", u32),
    ]


class MbTuning(C.Structure):
    _fields_ = [("digit_bits_max", u32), ("collide_block", u32), ("sort_algorithm", u32),
                ("frames_per_launch", u32), ("state_gather", u32), ("frame_kernel", u32),
                ("scatter_agents", u32), ("reserved", u32)]


MB_SORT_COUNTING, MB_SORT_ONESWEEP, MB_SORT_RANK = 0, 1, 2
MB_GATHER_COPY, MB_GATHER_INDIRECT = 0, 1
MB_FRAME_GRAPH, MB_FRAME_FUSED = 0, 1
MB_TUNE_CANDIDATES = 24
MB_BATCH_TUNE_CANDIDATES = 12


class MbServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("max_scenes", u32), ("max_agents", u32), ("max_cells", u32),
                ("reserved", u32 * 3)]


class MbServerStats(C.Structure):
    _fields_ = [("requests_done", C.c_uint64), ("frames", C.c_uint64), ("agent_steps", C.c_uint64),
                ("busy_seconds", C.c_double), ("scenes", u32), ("reserved", u32 * 3)]


MB_OK = 0
STATUS_NAMES = {
    0: "MB_OK",
    1: "MB_ERR_INVALID_ARG",
    2: "MB_ERR_OOM",
    3: "MB_ERR_CUDA",
    4: "MB_ERR_TIMEOUT",
    5: "MB_ERR_BUDGET_EXCEEDED",
    6: "MB_ERR_NOT_READY",
}
MB_HOST, MB_DEVICE = 0, 1

# name -> (restype, argtypes); every symbol declared in include/millionsball.h
SIGNATURES = {
    "mb_settings_default": (None, [C.POINTER(MbSettings)]),
    "mb_quantize_settings": (C.c_int, [C.POINTER(MbSettings), C.POINTER(MbConsts)]),
    "mb_create": (C.c_int, [C.POINTER(MbSettings), vp, C.POINTER(vp)]),
    "mb_destroy": (C.c_int, [vp]),
    "mb_set_settings": (C.c_int, [vp, C.POINTER(MbSettings)]),
    "mb_get_settings": (C.c_int, [vp, C.POINTER(MbSettings)]),
    "mb_set_state": (C.c_int, [vp, vp, vp, C.c_int]),
    "mb_get_state": (C.c_int, [vp, vp, vp, C.c_int]),
    "mb_step": (C.c_int, [vp, u32]),
    "mb_sync": (C.c_int, [vp]),
    "mb_get_debug": (C.c_int, [vp, vp, vp, vp, vp, C.c_int]),
    "mb_device_buffers": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "mb_time": (i64, [vp]),
    "mb_last_error": (C.c_char_p, [vp]),
    "mb_sort_plan_create": (C.c_int, [u32, u32, C.POINTER(vp)]),
    "mb_sort_plan_destroy": (C.c_int, [vp]),
    "mb_sort_and_hash": (C.c_int, [vp, vp, vp, u32, u32, vp, vp, vp, vp, vp]),
    "mb_sort_plan_status": (C.c_int, [vp, vp]),
    "mb_sort_plan_selftest_stall": (C.c_int, [vp, u32, vp]),
    "mb_sort_and_hash_static": (C.c_int, [vp, vp, u32, u32, vp, vp, vp, vp, vp]),
    "mb_sort_static_status": (C.c_int, [vp]),
    "mb_assemble_segments": (C.c_int, [vp, vp, u32, vp, vp, vp, vp]),
    "mb_render_topdown": (C.c_int, [vp, u32, u32, C.c_float, C.c_float, C.c_float, C.c_float, vp, vp, C.c_int]),
    "mb_render_view": (C.c_int, [vp, u32, u32, vp, vp, C.c_float, vp, vp, C.c_int]),
    "mb_get_tuning": (C.c_int, [vp, C.POINTER(MbTuning)]),
    "mb_set_tuning": (C.c_int, [vp, C.POINTER(MbTuning)]),
    "mb_autotune": (C.c_int, [vp, u32, C.POINTER(MbTuning), C.POINTER(C.c_float), C.POINTER(MbTuning)]),
    "mb_set_profiling": (C.c_int, [vp, C.c_int]),
    "mb_last_frame_times": (C.c_int, [vp, C.POINTER(C.c_float)]),
    "mb_kernels_per_frame": (u32, [vp]),
    "mb_batch_create": (C.c_int, [C.POINTER(MbSettings), u32, u32, u32, u32, vp, C.POINTER(vp)]),
    "mb_batch_add_scene": (C.c_int, [vp, C.POINTER(MbSettings), C.POINTER(u32)]),
    "mb_batch_destroy": (C.c_int, [vp]),
    "mb_batch_num_scenes": (u32, [vp]),
    "mb_batch_memory": (C.c_int, [vp, C.POINTER(C.c_uint64)]),
    "mb_batch_set_state": (C.c_int, [vp, u32, vp, vp, C.c_int]),
    "mb_batch_get_state": (C.c_int, [vp, u32, vp, vp, C.c_int]),
    "mb_batch_set_active": (C.c_int, [vp, u32, C.c_int]),
    "mb_batch_step": (C.c_int, [vp, u32]),
    "mb_batch_sync": (C.c_int, [vp]),
    "mb_batch_time": (i64, [vp, u32]),
    "mb_batch_get_debug": (C.c_int, [vp, u32, vp, vp, vp, vp, C.c_int]),
    "mb_batch_get_tuning": (C.c_int, [vp, C.POINTER(MbTuning)]),
    "mb_batch_set_tuning": (C.c_int, [vp, C.POINTER(MbTuning)]),
    "mb_batch_autotune": (C.c_int, [vp, u32, C.POINTER(MbTuning), C.POINTER(C.c_float), C.POINTER(MbTuning)]),
    "mb_server_create": (C.c_int, [C.POINTER(MbServerConfig), vp, C.POINTER(vp)]),
    "mb_server_destroy": (C.c_int, [vp]),
    "mb_server_submit_create": (C.c_int, [vp, C.POINTER(MbSettings), vp, vp, C.POINTER(u32), C.POINTER(C.c_uint64)]),
    "mb_server_submit_advance": (C.c_int, [vp, u32, u32, C.POINTER(C.c_uint64)]),
    "mb_server_wait": (C.c_int, [vp, C.c_uint64, C.c_double, C.POINTER(C.c_double)]),
    "mb_server_get_state": (C.c_int, [vp, u32, vp, vp]),
    "mb_server_get_stats": (C.c_int, [vp, C.POINTER(MbServerStats)]),
    "mb_selftest_divide": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]),
    "mb_version": (C.c_char_p, []),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libmillionsball.so (build it first with ``bevy_millions_ball_gb300.build``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"libmillionsball is not built ({p} missing); run "
            "`python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class MbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def check(lib: C.CDLL, status: int, world=None) -> None:
    if status != MB_OK:
        msg = lib.mb_last_error(world)
        raise MbError(status, (msg or b"").decode(errors="replace"))
