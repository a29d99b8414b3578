"""Loads the in-tree GB300 library and declares its C ABI (include/*.h)."""
import ctypes
import os

from . import build as _build

_HOST = None

VP = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double

# name -> (restype, argtypes); every symbol declared in include/gplum_p3t.h
# and include/p3t_tree.h
SIGNATURES = {
    # include/p3t_tree.h
    "p3t_tree_build": (VP, [I, VP, VP, VP, D, I, I]),
    "p3t_tree_status": (I, [VP]),
    "p3t_tree_counts": (None, [VP, VP]),
    "p3t_tree_export": (None, [VP, VP, VP, VP, VP, VP, VP, VP]),
    "p3t_tree_free": (None, [VP]),
    # include/gplum_p3t.h
    "p3t_init": (I, [I]),
    "p3t_finalize": (I, []),
    "p3t_set_params": (I, [VP]),
    "p3t_set_options": (I, [I, I, I]),
    "p3t_stream": (VP, []),
    "p3t_synchronize": (I, []),
    "p3t_epep": (I, [VP, I, VP, I, VP]),
    "p3t_epsp": (I, [VP, I, VP, I, VP]),
    "p3t_soft_dispatch": (I, [I, I, VP, VP, VP, VP, VP, VP]),
    "p3t_soft_retrieve": (I, [I, I, VP, VP]),
    "p3t_soft_dispatch_index": (I, [I, I, VP, VP, VP, VP, VP, VP, VP, I, VP, I, I]),
    "p3t_upload_particles": (I, [I, VP]),
    "p3t_upload_lists": (I, [I, VP, VP, VP, VP, VP, VP, VP, I]),
    "p3t_soft_run": (I, [I]),
    "p3t_download_forces": (I, [VP, I]),
    "p3t_status": (I, []),
    "p3t_soft_force_host": (I, [I, VP, I, VP, VP, VP, VP, VP, VP, VP, I, VP]),
    "p3t_probe_fma_peak": (I, [I, VP]),
    "p3t_snapshot_write_host": (I, [ctypes.c_char_p, I, VP, I, VP]),
    "p3t_snapshot_read_host": (I, [ctypes.c_char_p, I, VP, I, VP]),
    "p3t_snapshot_write": (I, [ctypes.c_char_p, I, VP, I]),
    "p3t_snapshot_wait": (I, []),
    "p3t_snapshot_read": (I, [ctypes.c_char_p, I, VP]),
    "p3t_collisions_write_host": (I, [ctypes.c_char_p, I, I, VP]),
    "p3t_collision_records": (I, [I, VP]),
    "p3t_collisions_write": (I, [ctypes.c_char_p, I]),
    "p3t_state_load": (I, [I, VP, VP, VP, VP, VP, VP]),
    "p3t_state_n": (I, []),
    "p3t_state_get": (I, [I, VP]),
    "p3t_state_set": (I, [I, VP]),
    "p3t_state_snapshot": (I, [I]),
    "p3t_set_cutoff_radii": (I, []),
    "p3t_set_r_planet": (I, []),
    "p3t_state_soft": (I, [I, VP, VP, VP, VP, VP, VP, VP, I]),
    "p3t_correct": (I, [I]),
    "p3t_neighbor_counts": (I, [VP, VP]),
    "p3t_neighbor_list": (I, [I, VP, I]),
    "p3t_neighbor_pairs": (I, [VP, ctypes.c_longlong]),
    "p3t_cluster_label": (I, []),
    "p3t_cluster_lists": (I, [VP, VP, VP]),
    "p3t_hard": (I, [I, I, VP, VP]),
    "p3t_set_hard_tiers": (I, [I, I]),
    "p3t_set_cluster_priority": (I, [VP, I]),
    "p3t_hard_costs": (I, [VP, I]),
    "p3t_hard_times": (I, [VP, I]),
    "p3t_set_hard_mode": (I, [I]),
    "p3t_set_fragmentation": (I, [D, I, D, ctypes.c_ulonglong]),
    "p3t_set_soft_tiles": (I, [I, I, I]),
    "p3t_set_soft_occupancy": (I, [I]),
    "p3t_set_hard_wide": (I, [I]),
    "p3t_set_hard_bundle": (I, [I, I]),
    "p3t_set_hard_heavy": (I, [ctypes.c_float]),
    "p3t_set_hard_lone": (I, [ctypes.c_float, I]),
    "p3t_set_walk": (I, [I]),
    "p3t_walk_last": (I, []),
    "p3t_set_walk_limits": (I, [I, ctypes.c_longlong]),
    "p3t_set_soft_pipe": (I, [I]),
    "p3t_set_hard_profile": (I, [I]),
    "p3t_hard_phase_cycles": (I, [VP, I]),
    "p3t_id_next": (ctypes.c_longlong, []),
    "p3t_mlp_set": (I, [VP, VP]),
    "p3t_mlp_get": (I, [VP, VP]),
    "p3t_mlp_reset": (I, []),
    "p3t_mlp_predict": (I, [VP, I, VP]),
    "p3t_mlp_loss_grad": (I, [VP, VP, I, VP, VP]),
    "p3t_mlp_train": (I, [VP, VP, I, I, I, ctypes.c_float, ctypes.c_ulonglong, VP]),
    "p3t_cluster_features": (I, [VP, I]),
    "p3t_set_schedule": (I, [I]),
    "p3t_state_tree": (I, [D, I, I]),
    "p3t_hard_enqueue": (I, []),
    "p3t_hard_integrate": (I, [I]),
    "p3t_hard_fetch": (I, [I, VP, VP]),
    "p3t_correct_and_search": (I, [I]),
    "p3t_remove_out_of_boundary": (I, [D, D, VP]),
    "p3t_state_tree_soft": (I, [D, I, I]),
    "p3t_tree_lists_counts": (I, [VP]),
    "p3t_tree_lists_get": (I, [VP] * 7),
    "p3t_kick": (I, []),
    "p3t_energy": (I, [VP]),
    "p3t_merge": (I, [VP]),
    "p3t_soft_force_noalloc": (I, [I, VP, I, VP, VP, VP, VP, VP, VP, VP, I, D, I, VP, VP]),
    "p3t_startup": (I, [VP, VP]),
    "p3t_tree_step": (I, [I, VP]),
    "p3t_step_phases_ms": (I, [VP]),
    "p3t_state_put_fpgrav": (I, [I, VP, ctypes.c_longlong]),
    "p3t_state_get_fpgrav": (I, [VP, I]),
    "p3t_set_hard_step_cap": (I, [I]),
    "p3t_hard_launch_stats": (I, [VP, VP, VP]),
    "p3t_launch_count": (ctypes.c_ulonglong, []),
}

# include/gplum_p3t.h: kernel status bits of the entry points that return a count
COUNT_STATUS_BASE = 65536


def status_bits(r):
    """The kernel status bits a count-returning entry point reported (0 if none)."""
    return -r - COUNT_STATUS_BASE if r <= -COUNT_STATUS_BASE else 0


def lib_path():
    return _build.LIB


def host_lib(build_if_missing=True):
    """The library handle.  Loading needs no GPU; compute calls do."""
    global _HOST
    if _HOST is not None:
        return _HOST
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(path)
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _HOST = lib
    return lib


def check(status, what):
    if status != 0:
        raise RuntimeError(f"{what} failed with status {status}")
