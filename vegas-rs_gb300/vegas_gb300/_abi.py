"""ctypes declarations of the C ABI in include/vegas_gpu.h.

The shared library is the only implementation: if it is missing or fails to
load, importing this module raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvegas_gpu.so")

VG_OK, VG_ERR_INVALID_ARG, VG_ERR_CUDA, VG_ERR_TIMEOUT, VG_ERR_OOM, VG_ERR_UNSUPPORTED, VG_ERR_NO_DEVICE = range(7)
SPIN_ISING, SPIN_HEISENBERG = 0, 1
CELL_SC, CELL_BCC, CELL_FCC = 0, 1, 2
PROPOSE_FLIP, PROPOSE_RANDOM = 0, 1
PATH_AUTO, PATH_GENERIC, PATH_STRUCTURED, PATH_RESIDENT, PATH_TILED = 0, 1, 2, 3, 4
FP32, FP64 = 0, 1


class LatticeDesc(C.Structure):
    _fields_ = [("cell", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("pbc_x", C.c_int32), ("pbc_y", C.c_int32), ("pbc_z", C.c_int32)]


class HamiltonianDesc(C.Structure):
    _fields_ = [("has_exchange", C.c_int32), ("exchange", C.c_double),
                ("has_anisotropy", C.c_int32), ("anisotropy", C.c_double), ("anisotropy_axis", C.c_double * 3),
                ("has_zeeman", C.c_int32), ("zeeman_sign", C.c_double),
                ("has_gauge", C.c_int32), ("gauge", C.c_double),
                ("has_cubic", C.c_int32), ("cubic", C.c_double),
                ("compound", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("spin_kind", C.c_int32), ("proposal", C.c_int32), ("path", C.c_int32),
                ("precision", C.c_int32), ("replica", C.c_uint32), ("threads_per_block", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("device", C.c_int32), ("max_device_bytes", C.c_int64)]


class Sums(C.Structure):
    _fields_ = [("bond", C.c_double), ("anisotropy", C.c_double), ("zeeman", C.c_double),
                ("cubic", C.c_double), ("mx", C.c_double), ("my", C.c_double), ("mz", C.c_double),
                ("accepted", C.c_double)]


class Info(C.Structure):
    _fields_ = [("n_sites", C.c_int64), ("n_colours", C.c_int32), ("coordination", C.c_int32),
                ("path", C.c_int32), ("precision", C.c_int32), ("grid_blocks", C.c_int32),
                ("threads_per_block", C.c_int32), ("sm_count", C.c_int32), ("device_bytes", C.c_int64),
                ("sweep_index", C.c_uint64)]


class ReplicaGroup(C.Structure):
    _fields_ = [("lattice", LatticeDesc), ("n_replicas", C.c_int32), ("temperatures", C.POINTER(C.c_double))]


class BatchInfo(C.Structure):
    _fields_ = [("n_groups", C.c_int32), ("total_replicas", C.c_int32), ("replica_words", C.c_int32),
                ("sweeps_per_round", C.c_int32), ("replica_sites", C.c_int64), ("sweep_index", C.c_uint64),
                ("round_index", C.c_uint32), ("graph", C.c_int32)]


class BatchTuning(C.Structure):
    _fields_ = [("threads_per_block", C.c_int32), ("words_per_thread", C.c_int32), ("words_in_flight", C.c_int32)]


class HeisReplica(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("replica", C.c_uint32), ("reserved", C.c_uint32),
                ("temperature", C.c_double), ("exchange", C.c_double), ("anisotropy", C.c_double),
                ("cubic", C.c_double)]


class HBatchDesc(C.Structure):
    _fields_ = [("lattice", LatticeDesc), ("anisotropy_axis", C.c_double * 3), ("field_axis", C.c_double * 3),
                ("zeeman_sign", C.c_double), ("precision", C.c_int32), ("proposal", C.c_int32)]


class HBatchInfo(C.Structure):
    _fields_ = [("n_replicas", C.c_int32), ("n_classes", C.c_int32), ("sites_per_replica", C.c_int64),
                ("sweep_index", C.c_uint64), ("sites_per_thread", C.c_int32), ("graph", C.c_int32),
                ("device_bytes", C.c_int64)]


HB_NSUMS = 12

# symbol -> (restype, argtypes); the list the header declares
P = C.POINTER
SIGNATURES = {
    "vg_status_string": (C.c_char_p, [C.c_int]),
    "vg_abi_version": (C.c_int, []),
    "vg_device_count": (C.c_int, [P(C.c_int32)]),
    "vg_device_name": (C.c_int, [C.c_int32, C.c_char_p, C.c_int32]),
    "vg_options_default": (C.c_int, [C.c_int32, P(Options)]),
    "vg_ctx_create": (C.c_int, [P(LatticeDesc), P(HamiltonianDesc), C.c_int32, C.c_uint64, P(C.c_void_p)]),
    "vg_ctx_create_ex": (C.c_int, [P(LatticeDesc), P(HamiltonianDesc), P(Options), C.c_uint64, P(C.c_void_p)]),
    "vg_ctx_destroy": (C.c_int, [C.c_void_p]),
    "vg_ctx_info": (C.c_int, [C.c_void_p, P(Info)]),
    "vg_last_error": (C.c_char_p, [C.c_void_p]),
    "vg_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vg_get_stream": (C.c_int, [C.c_void_p, P(C.c_void_p)]),
    "vg_init_random": (C.c_int, [C.c_void_p]),
    "vg_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "vg_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "vg_set_thermostat": (C.c_int, [C.c_void_p, C.c_double, P(C.c_double), C.c_double]),
    "vg_set_sweep_index": (C.c_int, [C.c_void_p, C.c_uint64]),
    "vg_get_sweep_index": (C.c_int, [C.c_void_p, P(C.c_uint64)]),
    "vg_sweeps": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int32, P(C.c_double), P(C.c_double)]),
    "vg_sweeps_sums": (C.c_int, [C.c_void_p, C.c_uint64, P(Sums)]),
    "vg_sweeps_async": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int32]),
    "vg_read_sums": (C.c_int, [C.c_void_p, C.c_uint64, P(Sums)]),
    "vg_synchronize": (C.c_int, [C.c_void_p]),
    "vg_time_passes": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int32, P(C.c_double), P(C.c_double)]),
    "vg_current_sums": (C.c_int, [C.c_void_p, P(Sums)]),
    "vg_total_energy": (C.c_int, [C.c_void_p, P(C.c_double)]),
    "vg_magnetization": (C.c_int, [C.c_void_p, P(C.c_double), P(C.c_double)]),
    "vg_energy_from_sums": (C.c_int, [C.c_void_p, P(Sums), P(C.c_double), P(C.c_double)]),
    "vg_batch_create": (C.c_int, [P(ReplicaGroup), C.c_int32, C.c_double, C.c_uint64, C.c_int32, C.c_int32,
                                  P(C.c_void_p)]),
    "vg_batch_destroy": (C.c_int, [C.c_void_p]),
    "vg_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "vg_batch_get_info": (C.c_int, [C.c_void_p, P(BatchInfo)]),
    "vg_batch_get_stream": (C.c_int, [C.c_void_p, P(C.c_void_p)]),
    "vg_batch_init_random": (C.c_int, [C.c_void_p]),
    "vg_batch_run": (C.c_int, [C.c_void_p, C.c_uint64]),
    "vg_batch_run_async": (C.c_int, [C.c_void_p, C.c_uint64]),
    "vg_batch_synchronize": (C.c_int, [C.c_void_p]),
    "vg_batch_observables": (C.c_int, [C.c_void_p, C.c_uint64, P(C.c_int64), P(C.c_int32)]),
    "vg_batch_ladder": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_int32)]),
    "vg_batch_swap_stats": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_int64), P(C.c_int64)]),
    "vg_batch_get_tuning": (C.c_int, [C.c_void_p, P(BatchTuning)]),
    "vg_batch_set_tuning": (C.c_int, [C.c_void_p, P(BatchTuning)]),
    "vg_batch_autotune": (C.c_int, [C.c_void_p, C.c_uint32, P(BatchTuning), P(C.c_double)]),
    "vg_batch_get_replica": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, P(C.c_int8)]),
    "vg_batch_set_replica": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, P(C.c_int8)]),
    "vg_hbatch_create": (C.c_int, [P(HBatchDesc), P(HeisReplica), C.c_int32, P(C.c_void_p)]),
    "vg_hbatch_destroy": (C.c_int, [C.c_void_p]),
    "vg_hbatch_last_error": (C.c_char_p, [C.c_void_p]),
    "vg_hbatch_get_info": (C.c_int, [C.c_void_p, P(HBatchInfo)]),
    "vg_hbatch_get_stream": (C.c_int, [C.c_void_p, P(C.c_void_p)]),
    "vg_hbatch_init_random": (C.c_int, [C.c_void_p]),
    "vg_hbatch_set_replica": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_double), C.c_int64]),
    "vg_hbatch_get_replica": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_double), C.c_int64]),
    "vg_hbatch_run": (C.c_int, [C.c_void_p, P(C.c_double), C.c_int32, C.c_uint32, C.c_uint32]),
    "vg_hbatch_run_async": (C.c_int, [C.c_void_p, P(C.c_double), C.c_int32, C.c_uint32, C.c_uint32]),
    "vg_hbatch_synchronize": (C.c_int, [C.c_void_p]),
    "vg_hbatch_point_sums": (C.c_int, [C.c_void_p, P(C.c_double), C.c_int64]),
    "vg_hbatch_time_passes": (C.c_int, [C.c_void_p, C.c_uint32, P(C.c_double)]),
    "vg_ising_sc_sweeps_noalloc": (C.c_int, [P(LatticeDesc), C.c_double, C.c_double, C.c_double, C.c_uint64,
                                             C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p]),
    "vg_wolff_steps": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int32, P(C.c_double), P(C.c_double)]),
    "vg_selftest_grid_barrier": (C.c_int, [C.c_void_p, C.c_int32]),
    "vg_set_exchange_bonds": (C.c_int, [C.c_void_p, P(C.c_double), C.c_int64]),
    "vg_site_energies": (C.c_int, [C.c_void_p, P(C.c_double), C.c_int64]),
    "vg_delta_energies": (C.c_int, [C.c_void_p, P(C.c_double), P(C.c_double), C.c_int64]),
    "vg_lattice_neighbours": (C.c_int, [P(LatticeDesc), P(C.c_int32), C.c_int64, P(C.c_int64), P(C.c_int32)]),
    "vg_lattice_colouring": (C.c_int, [P(LatticeDesc), P(C.c_int32), C.c_int64, P(C.c_int32)]),
    "vg_host_alloc": (C.c_int, [P(C.c_void_p), C.c_uint64]),
    "vg_host_free": (C.c_int, [C.c_void_p]),
}


def load(path: str = "") -> C.CDLL:
    """Load the library (VEGAS_GPU_LIB overrides the in-tree build's path)."""
    path = path or os.environ.get("VEGAS_GPU_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first (__graft_entry__.build())")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


class VegasGpuError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
