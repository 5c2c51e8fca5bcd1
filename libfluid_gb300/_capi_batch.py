"""ctypes signatures of the batched and served entry points of include/sph_c.h."""
import ctypes as C

from ._capi import SphParams

_P, _I, _U32, _F = C.c_void_p, C.c_int, C.c_uint32, C.c_float


class SphLattice(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("spacing", C.c_float), ("nx", C.c_uint32), ("ny", C.c_uint32),
                ("nz", C.c_uint32), ("jitter", C.c_float), ("vel", C.c_float * 3), ("pad_", C.c_uint32),
                ("seed", C.c_uint64)]


SIGNATURES = [
    ("sph_batch_create", _I, [C.POINTER(_P), _I]),
    ("sph_batch_destroy", _I, [_P]),
    ("sph_batch_add_scene", _I, [_P, C.POINTER(SphParams), _U32, C.POINTER(_I)]),
    ("sph_batch_remove_scene", _I, [_P, _I]),
    ("sph_batch_set_params", _I, [_P, _I, C.POINTER(SphParams)]),
    ("sph_batch_set_boundary", _I, [_P, _I, _I]),
    ("sph_batch_set_state", _I, [_P, _I, _P, _P, _U32]),
    ("sph_batch_generate_lattice", _I, [_P, _I, C.POINTER(SphLattice), _U32]),
    ("sph_batch_step", _I, [_P, _U32]),
    ("sph_batch_step_async", _I, [_P, _U32]),
    ("sph_batch_sync", _I, [_P]),
    ("sph_batch_get_state", _I, [_P, _I, _P, _P, _P, _U32]),
    ("sph_batch_snapshot", _I, [_P, _I, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("sph_batch_restore", _I, [_P, _I, _P, C.c_uint64]),
    ("sph_batch_num_scenes", _U32, [_P]),
    ("sph_batch_num_particles", C.c_uint64, [_P]),
    ("sph_batch_debug_enable", _I, [_P, _I]),
    ("sph_batch_debug_get", _I, [_P, _I, _I, _P, C.c_uint64]),
    ("sph_batch_set_use_graph", _I, [_P, _I]),
    ("sph_batch_set_exec", _I, [_P, _P]),
    ("sph_batch_set_deferred_xsph", _I, [_P, _I]),
    ("sph_batch_timer_mark", _I, [_P, _I]),
    ("sph_batch_set_profiling", _I, [_P, _I]),
    ("sph_batch_get_pass_times", _I, [_P, C.POINTER(C.c_double), _I, C.POINTER(C.c_uint64)]),
    ("sph_batch_timer_elapsed", _I, [_P, _I, _I, C.POINTER(_F)]),
    ("sph_batch_last_error", C.c_char_p, [_P]),
    ("sph_server_create", _I, [C.POINTER(_P), _P]),
    ("sph_server_destroy", _I, [_P]),
    ("sph_server_submit", _I, [_P, _P, C.POINTER(C.c_uint64)]),
    ("sph_server_state", _I, [_P, C.c_uint64]),
    ("sph_server_wait", _I, [_P, C.c_uint64, C.c_int64]),
    ("sph_server_fetch", _I, [_P, C.c_uint64, _P, _P, _U32]),
    ("sph_server_times", _I, [_P, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.POINTER(C.c_double)]),
    ("sph_server_get_stats", _I, [_P, _P]),
    ("sph_server_drain", _I, [_P, C.c_int64]),
    ("sph_server_last_error", C.c_char_p, [_P]),
]
