"""ctypes binding of libxdem's C ABI (include/xdem.h).

Loading fails loudly when the library has not been built; there is no CPU or
PyTorch fallback for any compute call.  Device pointers are passed as plain
integers (e.g. ``tensor.data_ptr()``); the stream is a ``cudaStream_t``
(``torch.cuda.current_stream().cuda_stream``) or 0 for the legacy stream.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libxdem.so")

vp = C.c_void_p
u32 = C.c_uint
i32 = C.c_int
u64 = C.c_ulonglong
szt = C.c_size_t

XD_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
          4: "capacity exceeded", 5: "device wait timed out", 6: "call out of order"}


class XdemError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed: {STATUS.get(status, status)} ({msg})")
        self.status = status


# name -> argtypes (restype int unless listed in _RESTYPES)
_SIGS = {
    "xd_version": [],
    "xd_status_string": [i32],
    "xd_last_error": [C.c_char_p, szt],
    "xd_clear_error": [],
    "xd_sizeof": [C.c_char_p],
    "xd_release_workspace": [],
    "xd_report_unsupported": [C.c_char_p],
    "xd_set_symbolic_parameter": [vp],
    "xd_vv_update_position": [vp, vp, vp, u32, vp],
    "xd_vv_update_velocity": [vp] * 8 + [u32, vp],
    "xd_vv_update_velocity_position": [vp] * 9 + [u32, vp],
    "xd_calculate_hash_and_index": [vp, vp, vp, u32, vp],
    "xd_calculate_hash_and_index_polysphere": [vp, vp, u32, u32, vp, vp],
    "xd_reorder_and_find_cell_start": [vp] * 5 + [u32, u32, vp],
    "xd_reorder_and_find_cell_start_noalloc": [vp] * 5 + [u32, u32, vp],
    "xd_radix_sort_pairs": [vp, vp, u32, u32, vp],
    "xd_calculate_p2p": [i32] + [vp] * 10 + [u32, vp],
    "xd_plane_contact_force": [i32] + [vp] * 7 + [u32, vp, vp],
    "xd_cube_contact_force": [i32] + [vp] * 7 + [u32, vp, vp],
    "xd_cylinder_contact_force": [i32] + [vp] * 7 + [u32] + [vp] * 5,
    "xd_planes_contact_force": [i32, vp, vp, u32] + [vp] * 6 + [u32, vp],
    "xd_particle_polygon_collision": [i32] + [vp] * 13 + [u32, u32, vp],
    "xd_set_symbolic_parameter_f": [vp],
    "xd_vv_update_position_f": [vp, vp, vp, u32, vp],
    "xd_vv_update_velocity_f": [vp] * 8 + [u32, vp],
    "xd_calculate_hash_and_index_f": [vp, vp, vp, u32, vp],
    "xd_calculate_hash_and_index_polysphere_f": [vp, vp, u32, u32, vp, vp],
    "xd_reorder_and_find_cell_start_f": [vp] * 5 + [u32, u32, vp],
    "xd_calculate_p2p_f": [i32] + [vp] * 10 + [u32, vp],
    "xd_plane_contact_force_f": [i32] + [vp] * 7 + [u32, vp, vp],
    "xd_cube_contact_force_f": [i32] + [vp] * 7 + [u32, vp, vp],
    "xd_particle_polygon_collision_f": [i32] + [vp] * 13 + [u32, u32, vp],
    "xd_reduction_f3": [vp, u32, vp, vp],
    "xd_legacy_set_symbolic_parameter": [vp],
    "xd_legacy_vv_update_position": [vp, vp, vp, u32, vp],
    "xd_legacy_vv_update_velocity": [vp] * 6 + [u32, vp],
    "xd_legacy_calculate_hash_and_index": [vp, vp, vp, u32, vp],
    "xd_legacy_reorder_and_find_cell_start": [vp] * 5 + [u32, u32, vp],
    "xd_legacy_calculate_p2p": [vp] * 10 + [u32, u32, vp],
    "xd_legacy_cube_hertzian_contact_force": [vp] + [C.c_double] * 5 + [vp] * 6 + [u32, vp],
    "xd_legacy_shape_hertzian_contact_force": [vp] * 5 + [C.c_double] * 5 + [vp] * 7 + [u32] + [vp] * 5,
    "xd_legacy_update_polygons_position": [vp, vp, vp, u32, vp, vp],
    "xd_legacy_update_polygons_information": [vp, vp, vp, u32, vp],
    "xd_legacy_mergedata": [vp, vp, u32, vp, u32, vp],
    "xd_update_polygon_object_data": [vp] * 4 + [u32, vp],
    "xd_reduction_d3": [vp, u32, vp, vp],
    "xd_pair_list": [vp] * 4 + [u32, vp, vp, u64, vp, vp],
    "xd_scene_create": [vp, vp],
    "xd_scene_destroy": [vp],
    "xd_scene_upload": [vp] * 10 + [vp],
    "xd_scene_download": [vp] * 8 + [vp],
    "xd_scene_upload_async": [vp] * 10 + [vp],
    "xd_scene_download_async": [vp] * 8 + [vp],
    "xd_scene_device_state": [vp] * 10,
    "xd_scene_device_grid": [vp] * 6,
    "xd_scene_download_grid": [vp] * 6 + [vp],
    "xd_scene_set_bodies": [vp, vp, vp],
    "xd_scene_get_bodies": [vp, vp, vp],
    "xd_scene_step": [vp, u32, i32, vp],
    "xd_scene_launches": [vp, u32],
    "xd_scene_set_timing": [vp, i32],
    "xd_scene_eval_contacts": [vp, vp, vp, vp],
    "xd_scene_pair_list": [vp, u32, vp, vp, vp],
    "xd_scene_counters": [vp, vp, vp],
    "xd_scene_stats": [vp, vp, u32, vp],
    "xd_scene_set_tuning": [vp, vp],
    "xd_scene_get_tuning": [vp, vp],
    "xd_scene_rebuilds": [vp, vp, vp, vp],
    "xd_scene_step_many": [vp, vp, u32, i32, vp],
    "xd_scene_set_tangential_history": [vp, u32],
    "xd_scene_set_particle_grid": [vp, vp, C.c_double, vp],
    "xd_scene_set_kinematic_bodies": [vp, i32],
    "xd_scene_set_emitter": [vp, u32, u32, vp, u32, vp],
    "xd_scene_set_planes": [vp, vp, vp],
    "xd_batch_create": [vp, u32, vp],
    "xd_batch_step": [vp, u32, i32, vp],
    "xd_batch_destroy": [vp],
    "xd_batch_set_timing": [vp, i32],
    "xd_batch_kernel_times": [vp, vp, vp],
    "xd_scene_active": [vp, vp],
    "xd_scene_download_history": [vp, vp, vp, vp, vp],
    "xd_scene_device_bytes": [vp, vp],
    "xd_scene_phase_times": [vp, vp, vp],
}
_RESTYPES = {"xd_version": C.c_char_p, "xd_status_string": C.c_char_p, "xd_clear_error": None,
             "xd_sizeof": szt, "xd_scene_launches": u64}

_lib = None


def lib() -> C.CDLL:
    """The loaded libxdem (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} not found: build libxdem first "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPES.get(name, i32)
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def call(name: str, *args) -> int:
    """Call an int-returning ABI function; raise XdemError on a non-OK status."""
    L = lib()
    st = getattr(L, name)(*args)
    if st != XD_OK:
        buf = C.create_string_buffer(512)
        L.xd_last_error(buf, 512)
        L.xd_clear_error()
        raise XdemError(name, st, buf.value.decode(errors="replace"))
    return st


def ptr(x) -> int:
    """Device (or host) address of a torch tensor / numpy array / int / None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")
