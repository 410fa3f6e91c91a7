"""ctypes binding of the C ABI declared in ``include/particulator_gb300.h``.

The library is the in-tree ``_build/libparticulator_gb300.so``.  There is no
fallback: if it is missing, ``lib()`` raises, and every device entry point
returns ``PCL_ERR_CUDA`` when no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# PCL_LIB_PATH selects another build of the same library (e.g. a variant built
# with different compile-time options); the default is the in-tree build.
LIB_PATH = os.environ.get("PCL_LIB_PATH") or os.path.join(HERE, "_build", "libparticulator_gb300.so")

PCL_OK = 0
PCL_ERR_INVALID = -1
PCL_ERR_CUDA = -2
PCL_ERR_CAPACITY = -3
PCL_ERR_UNSUPPORTED = -4
PCL_ERR_STATE = -5
PCL_ERR_TIMEOUT = -6
HOST_IO_AUTO, HOST_IO_COPY, HOST_IO_DIRECT = 0, 1, 2
PCL_ERR_NUMERIC = -7
NOALLOC_MAX_SLOTS = 1 << 25

ELECTRON, PHOTON, POSITRON = 0, 1, 2
SPECIES_TRACKED, SPECIES_TALLY_ONLY = 0, 1

PROC_MOLLER = 1
PROC_RBEB = 2
PROC_SELTZER_BERGER = 3
PROC_REL_COULOMB = 4
PROC_COMPTON = 5
PROC_KN_COMPTON = 6
PROC_PHOTOELECTRIC = 7
PROC_BETHE_HEITLER = 8
PROC_BHABHA = 9
PROC_ANNIHILATION = 10
PROC_ELASTIC = 11
PROC_EXCITATION = 12
PROC_NULL_COLLISION = 13
PROC_IONIZATION = 14
PROC_ATTACHMENT = 15

MAX_PROC = 16
NERR = 8
ERROR_NAMES = ["ratebound", "table_range", "reject_cap", "substep_cap", "spill", "capacity",
               "kinematics", "neg_rate"]

_P = C.POINTER
_d = C.c_double
_i32 = C.c_int32
_i64 = C.c_int64
_u64 = C.c_uint64
_u32 = C.c_uint32


class Process(C.Structure):
    _fields_ = [("kind", _i32), ("Z", _i32), ("coef", _d), ("param", _d * 8), ("nparam", _i32),
                ("naux", _i32), ("aux0", _P(_d)), ("aux1", _P(_d)), ("aux2", _P(_d)), ("naux2", _i32),
                ("reserved", _i32)]


class Config(C.Structure):
    _fields_ = [("seed", _u64), ("device", _i32), ("block_size", _i32), ("grid_blocks", _i32),
                ("steps_per_launch", _i32), ("compaction_period", _i32), ("use_graph", _i32),
                ("blocks_per_sm", _i32), ("classic_step", _i32), ("stash_entries", _i32), ("reserved", _i32)]


class Tallies(C.Structure):
    _fields_ = [("t", _d), ("steps", _i64), ("n", _i64 * 3), ("live", _i64 * 3), ("particle_steps", _i64),
                ("collisions", (_i64 * MAX_PROC) * 3), ("nulls", _i64 * 3), ("spawned", _i64 * 3),
                ("tally_count", _i64 * 3), ("tally_w", _d * 3), ("tally_wE", _d * 3), ("errors", _i64 * NERR)]


class RunOpts(C.Structure):
    _fields_ = [("target_species", _i32), ("target_ismax", _i32), ("target_n", _i64), ("max_steps", _i64)]


class TuneResult(C.Structure):
    _fields_ = [("blocks_per_sm", _i32), ("steps_per_launch", _i32), ("compaction_period", _i32),
                ("use_graph", _i32), ("rate", _d), ("trials", _i32), ("steps", _i32), ("reserved", _i32 * 2)]


class Packed(C.Structure):
    _fields_ = [("xw", _P(C.c_float)), ("ps", _P(C.c_float)), ("meta", _P(_u32))]


_SIGS = {
    "pcl_sb_build": (C.c_int, [C.c_int, C.c_int, C.c_int, _P(_d), _P(_d), _P(_d), C.c_int, _d, _d, _d,
                               _P(_d), _P(_d), _P(_d)]),
    "pcl_totalcs": (C.c_int, [_P(Process), _i64, _P(_d), _P(_d)]),
    "pcl_build_collision_table": (C.c_int, [C.c_int, C.c_int, _P(Process), _d, _d, C.c_int, C.c_int, _d,
                                            _P(_d), _P(_d), _P(_i32)]),
    "pcl_ratebound_split": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _d, _P(_d), _d, _P(_d), _P(_d)]),
    "pcl_build_continuum_loss": (C.c_int, [_d, _d, _d, _d, C.c_int, _P(C.c_int), _P(_d), _P(_d), _P(_d),
                                           C.c_int]),
    "pcl_create": (C.c_int, [_P(Config), _P(C.c_void_p)]),
    "pcl_destroy": (None, [C.c_void_p]),
    "pcl_last_error": (C.c_char_p, [C.c_void_p]),
    "pcl_version": (C.c_char_p, []),
    "pcl_device_count": (C.c_int, []),
    "pcl_set_species": (C.c_int, [C.c_void_p, C.c_int, _d, _i64, C.c_int]),
    "pcl_set_collision_table": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _d, _P(_d), _P(_d),
                                          _P(Process)]),
    "pcl_set_linear_table": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _d, _d, _P(_d), _P(_d), C.c_int,
                                       _P(Process)]),
    "pcl_set_forcing": (C.c_int, [C.c_void_p, _P(_d), _P(_d), C.c_int, C.c_int, _d, _P(_d), _P(_d)]),
    "pcl_set_field": (C.c_int, [C.c_void_p, C.c_int, _P(_d), C.c_int]),
    "pcl_set_push_mask": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "pcl_set_bfield": (C.c_int, [C.c_void_p, C.c_int, _P(_d), C.c_int]),
    "pcl_roulette": (C.c_int, [C.c_void_p, C.c_int, _d]),
    "pcl_split": (C.c_int, [C.c_void_p, C.c_int, _d]),
    "pcl_roulette_fn": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(_d), _P(_d)]),
    "pcl_split_fn": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(_d), _P(_d)]),
    "pcl_roulette_swarms": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(_d)]),
    "pcl_set_wall": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _d, C.c_int, _i64]),
    "pcl_get_wall": (C.c_int, [C.c_void_p, _P(_i64), _P(_i32), _P(_u64), _P(_d), _P(_d), _P(_d), _P(_d)]),
    "pcl_set_swarms": (C.c_int, [C.c_void_p, C.c_int, _P(_d), _P(_d), _d]),
    "pcl_swarm_moments": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(_d)]),
    "pcl_swarm_counts": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(_i64)]),
    "pcl_energy_histogram": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _P(_d), _P(_i64), _P(_d)]),
    "pcl_set_swarm_cap": (C.c_int, [C.c_void_p, C.c_int, _i64]),
    "pcl_upload": (C.c_int, [C.c_void_p, C.c_int, _i64, _P(_d), _P(_d), _P(_d), _P(_d), _P(_d), _P(_u64),
                             _u64]),
    "pcl_download": (C.c_int, [C.c_void_p, C.c_int, _P(_i64), _P(_d), _P(_d), _P(_d), _P(_d), _P(_d),
                               _P(_u64), _P(_u32)]),
    "pcl_upload_packed": (C.c_int, [C.c_void_p, C.c_int, _i64, _P(Packed)]),
    "pcl_advance_host": (C.c_int, [C.c_void_p, _d, _P(_i64), _P(Packed), _P(_i64), _P(Packed), _P(_i64), C.c_int,
                                   C.c_int]),
    "pcl_host_register": (C.c_int, [C.c_void_p, C.c_size_t]),
    "pcl_host_unregister": (C.c_int, [C.c_void_p]),
    "pcl_host_alloc": (C.c_int, [_P(C.c_void_p), C.c_size_t]),
    "pcl_host_free": (C.c_int, [C.c_void_p]),
    "pcl_test_timeout": (C.c_int, [C.c_void_p, C.c_int]),
    "pcl_download_packed": (C.c_int, [C.c_void_p, C.c_int, _P(_i64), _P(Packed)]),
    "pcl_advance": (C.c_int, [C.c_void_p, _d]),
    "pcl_run": (C.c_int, [C.c_void_p, _d, _d, _P(RunOpts), _P(Tallies)]),
    "pcl_get_tallies": (C.c_int, [C.c_void_p, _P(Tallies)]),
    "pcl_reset_tallies": (C.c_int, [C.c_void_p]),
    "pcl_moments": (C.c_int, [C.c_void_p, C.c_int, _P(_d)]),
    "pcl_compact": (C.c_int, [C.c_void_p]),
    "pcl_set_tally_histogram": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _d, _d]),
    "pcl_get_tally_histogram": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(_i64), _P(_d)]),
    "pcl_sync": (C.c_int, [C.c_void_p]),
    "pcl_timer_start": (C.c_int, [C.c_void_p]),
    "pcl_timer_stop": (C.c_int, [C.c_void_p, _P(_d)]),
    "pcl_kernel_stats": (C.c_int, [C.c_void_p, _P(_d), _P(_i64), _P(_i64), _P(_d), C.c_int]),
    "pcl_compact_noalloc": (C.c_int, [_i64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
    "pcl_test_sampler": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _i64, _P(_d), _P(_u64), _P(_d), _P(_d),
                                   _P(_i32), _P(_u32)]),
    "pcl_mlp_create": (C.c_int, [C.c_int, _u64, _P(C.c_void_p)]),
    "pcl_mlp_destroy": (None, [C.c_void_p]),
    "pcl_mlp_last_error": (C.c_char_p, [C.c_void_p]),
    "pcl_mlp_set_params": (C.c_int, [C.c_void_p, _P(C.c_float), _i64]),
    "pcl_mlp_get_params": (C.c_int, [C.c_void_p, _P(C.c_float), _i64]),
    "pcl_mlp_forward": (C.c_int, [C.c_void_p, _i64, _P(C.c_float), _P(C.c_float)]),
    "pcl_mlp_gradient": (C.c_int, [C.c_void_p, _i64, _P(C.c_float), _P(C.c_float), _P(C.c_float), _P(_d)]),
    "pcl_mlp_train": (C.c_int, [C.c_void_p, _i64, _P(C.c_float), _P(C.c_float), _i64, _i32, _d, _u64, _P(_d)]),
    "pcl_set_learned": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "pcl_autotune": (C.c_int, [C.c_void_p, _d, _i32, _P(TuneResult)]),
    "pcl_set_launch": (C.c_int, [C.c_void_p, _i32, _i32, _i32, _i32]),
    "pcl_set_host_io": (C.c_int, [C.c_void_p, C.c_int]),
    "pcl_time_energy_draw": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, _i64, C.c_int, _P(_d),
                                       _P(_d), _P(C.c_float), _P(C.c_float), _P(C.c_uint32)]),
    "pcl_learn_stats": (C.c_int, [C.c_void_p, _P(_i64), _P(_i64)]),
    "pcl_learn_data": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _i64, C.c_int, _u64,
                                 _P(C.c_float), _P(C.c_float), _P(_i64)]),
}

MLP_NPARAM = 33537

_lib = None


def lib():
    """Load the shared library once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} not found: build it first (python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


class PCLError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"particulator_gb300 error {code}: {msg}")
        self.code = code


def check(rc, ctx=None, what=""):
    if rc != PCL_OK:
        msg = ""
        if ctx:
            msg = lib().pcl_last_error(ctx).decode(errors="replace")
        raise PCLError(rc, f"{what}: {msg}" if what else msg)
    return rc


def dptr(a):
    """Pointer to a contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_P(_d))


def u64ptr(a):
    return None if a is None else a.ctypes.data_as(_P(_u64))


def u32ptr(a):
    return None if a is None else a.ctypes.data_as(_P(_u32))


def i32ptr(a):
    return None if a is None else a.ctypes.data_as(_P(_i32))


def fptr(a):
    """Pointer to a contiguous float32 numpy array (or None)."""
    return None if a is None else a.ctypes.data_as(_P(C.c_float))


def i64ptr(a):
    return None if a is None else a.ctypes.data_as(_P(_i64))
