"""ctypes binding of the C ABI declared in include/uppasd_gpu.h.

The shared library is the product: there is no CPU fallback.  Loading fails
with an explicit error when ``libuppasd_gb300.so`` has not been built, and
every call that returns a negative status raises ``UppasdGpuError`` carrying
``uppasd_gpu_last_error()``.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libuppasd_gb300.so")

I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)


class UppasdGpuError(RuntimeError):
    def __init__(self, fn, rc, msg):
        super().__init__(f"{fn} failed with status {rc}: {msg}")
        self.rc = rc


class Consts(C.Structure):
    _fields_ = [
        ("natom", C.c_int32), ("mensemble", C.c_int32), ("max_no_neigh", C.c_int32), ("nham", C.c_int32),
        ("do_dm", C.c_int32), ("max_no_dmneigh", C.c_int32), ("do_aniso", C.c_int32), ("sdealgh", C.c_int32),
        ("delta_t", C.c_double), ("bn", C.c_double), ("temprescale", C.c_double),
        ("gpu_rng_seed", C.c_uint64), ("gpu_rng", C.c_int32), ("precision", C.c_int32),
        ("n1", C.c_int32), ("n2", C.c_int32), ("n3", C.c_int32), ("na", C.c_int32),
    ]


class Arrays(C.Structure):
    _fields_ = [
        ("nlist", I32P), ("nlistsize", I32P), ("ncoup", F64P), ("aham", I32P),
        ("dmlist", I32P), ("dmlistsize", I32P), ("dm_vect", F64P),
        ("taniso", I32P), ("eaniso", F64P), ("kaniso", F64P), ("sb", F64P),
        ("external_field", F64P), ("mmom", F64P), ("lambda1_array", F64P), ("temp_array", F64P),
        ("landeg", F64P), ("emom", F64P), ("species", I32P),
    ]


# uppasd_gpu_measure_cb: (step, emom, emomM, user) -> int
MEASURE_CB = C.CFUNCTYPE(C.c_int, C.c_int64, F64P, F64P, C.c_void_p)

# name -> (argtypes) ; all return int status
SIGNATURES = {
    "uppasd_gpu_device_info": [I32P, I32P, I32P, C.POINTER(C.c_int64)],
    "uppasd_gpu_init": [C.POINTER(Consts), C.POINTER(Arrays), C.POINTER(C.c_void_p)],
    "uppasd_gpu_finalize": [C.c_void_p],
    "uppasd_gpu_put_moments": [C.c_void_p, F64P],
    "uppasd_gpu_get_moments": [C.c_void_p, F64P, F64P],
    "uppasd_gpu_set_temperature": [C.c_void_p, F64P],
    "uppasd_gpu_set_step": [C.c_void_p, C.c_int64],
    "uppasd_gpu_set_jtensor": [C.c_void_p, F64P],
    "uppasd_gpu_set_dipole": [C.c_void_p, C.c_int32, C.c_double, F64P, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                              F64P, F64P],
    "uppasd_gpu_set_relaxtime": [C.c_void_p, C.c_double],
    "uppasd_gpu_set_units": [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double],
    "uppasd_gpu_set_perp": [C.c_void_p, C.c_int32],
    "uppasd_gpu_set_noise": [C.c_void_p, F64P, C.c_int64],
    "uppasd_gpu_sd_run": [C.c_void_p, C.c_int64],
    "uppasd_gpu_sd_run_io": [C.c_void_p, F64P, C.c_int64, F64P, F64P],
    "uppasd_gpu_sd_run_measured": [C.c_void_p, C.c_int64, C.c_int64, MEASURE_CB, C.c_void_p],
    "uppasd_gpu_get_field": [C.c_void_p, F64P],
    "uppasd_gpu_mc_run": [C.c_void_p, C.c_char, C.c_double, C.c_int64],
    "uppasd_gpu_observables": [C.c_void_p, F64P, F64P, F64P],
    "uppasd_gpu_energy_terms": [C.c_void_p, F64P],
    "uppasd_gpu_mc_run_square": [C.c_void_p, C.c_int32, C.c_double, C.c_int64],
    "uppasd_gpu_mc_run_square_temps": [C.c_void_p, C.c_int32, F64P, C.c_int64],
    "uppasd_gpu_mc_run_temps": [C.c_void_p, C.c_char, F64P, C.c_int64],
    "uppasd_gpu_pt_run": [C.c_void_p, F64P, C.c_int64, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                          I32P],
    "uppasd_gpu_set_stream": [C.c_void_p, C.c_void_p],
    "uppasd_gpu_time_kernels": [C.c_void_p, C.c_int32, F64P],
    "uppasd_gpu_path_info": [C.c_void_p, C.POINTER(C.c_int64)],
    "uppasd_gpu_moment_sums_noalloc": [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p],
    # batched replica Monte Carlo
    "uppasd_gpu_mcbatch_create": [C.c_int32, I32P, F64P, I32P, F64P, C.c_double, F64P, C.c_uint64, C.c_int32,
                                  C.c_int32, C.POINTER(C.c_void_p)],
    "uppasd_gpu_mcbatch_destroy": [C.c_void_p],
    "uppasd_gpu_mcbatch_set_stream": [C.c_void_p, C.c_void_p],
    "uppasd_gpu_mcbatch_set_schedule": [C.c_void_p, C.c_int32, C.c_int32, I32P],
    "uppasd_gpu_mcbatch_get_schedule": [C.c_void_p, I32P, I32P, I32P],
    "uppasd_gpu_mcbatch_autotune": [C.c_void_p, C.c_int32, C.c_char_p, C.POINTER(C.c_float)],
    "uppasd_gpu_mcbatch_run": [C.c_void_p, C.c_int64, C.c_int32, C.c_int32],
    "uppasd_gpu_mcbatch_enqueue": [C.c_void_p, C.c_int64, C.c_int32, C.c_int32],
    "uppasd_gpu_mcbatch_check": [C.c_void_p],
    "uppasd_gpu_mcbatch_stats": [C.c_void_p, F64P, C.POINTER(C.c_int64), F64P],
    "uppasd_gpu_mcbatch_series": [C.c_void_p, F64P],
    "uppasd_gpu_mcbatch_reset_stats": [C.c_void_p],
    "uppasd_gpu_mcbatch_get_spins": [C.c_void_p, F64P],
    "uppasd_gpu_mcbatch_put_spins": [C.c_void_p, F64P],
    "uppasd_gpu_mcbatch_set_sweep": [C.c_void_p, C.c_int64],
    "uppasd_gpu_mcbatch_set_exchange": [C.c_void_p, C.c_int32],
    "uppasd_gpu_mcbatch_exchange_state": [C.c_void_p, I32P, I32P, I32P, C.POINTER(C.c_int64),
                                          C.POINTER(C.c_int64)],
    "uppasd_gpu_mcbatch_set_replica_ids": [C.c_void_p, C.c_int32],
    "uppasd_gpu_mcbatch_set_spin_limit": [C.c_void_p, C.c_int64],
    "uppasd_gpu_tc_wait_selftest": [],
    # tcgen05 BF16 GEMM on host buffers (validation entry point)
    "uppasd_gpu_tc_gemm": [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                           C.c_int32, C.c_int32, C.c_void_p, C.c_void_p],
    # learned patch proposal
    "uppasd_gpu_proposal_create": [C.c_void_p, C.c_int32, C.c_float, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)],
    "uppasd_gpu_proposal_destroy": [C.c_void_p],
    "uppasd_gpu_proposal_nparams": [C.c_void_p, C.POINTER(C.c_int64)],
    "uppasd_gpu_proposal_get_params": [C.c_void_p, C.c_void_p],
    "uppasd_gpu_proposal_set_params": [C.c_void_p, C.c_void_p],
    "uppasd_gpu_proposal_get_masks": [C.c_void_p, C.c_void_p],
    "uppasd_gpu_proposal_forward": [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p],
    "uppasd_gpu_proposal_loss_grad": [C.c_void_p, C.c_void_p, C.c_int32, F64P, C.c_void_p],
    "uppasd_gpu_proposal_collect": [C.c_void_p],
    "uppasd_gpu_proposal_train": [C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_void_p],
    "uppasd_gpu_proposal_sweep": [C.c_void_p, C.c_double, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  F64P],
    "uppasd_gpu_proposal_mix": [C.c_void_p, C.c_double, C.c_int64, C.c_int32, C.POINTER(C.c_int64),
                                C.POINTER(C.c_int64), F64P],
    "uppasd_gpu_proposal_mix_temps": [C.c_void_p, F64P, C.c_int64, C.c_int32, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64), F64P],
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the CUDA library; raise if it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()'). "
            "The GB300 hot path has no CPU fallback.")
    lib = C.CDLL(path)
    lib.uppasd_gpu_last_error.restype = C.c_char_p
    lib.uppasd_gpu_last_error.argtypes = []
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    _lib = lib
    return lib


def exported_symbols():
    return ["uppasd_gpu_last_error", *SIGNATURES]


def call(name, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.uppasd_gpu_last_error()
        raise UppasdGpuError(name, rc, msg.decode() if msg else "")
    return rc
