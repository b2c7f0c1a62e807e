"""ctypes mirror of the C ABI in include/ismc.h.

The struct layouts here are checked against the library's own ``ismc_sizeof``
when the library is loaded, so a mismatch fails loudly instead of corrupting
memory.
"""
import ctypes as C

MAXL = 16
ABI_VERSION = 1

OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_STEP_LIMIT = -3
ERR_NO_DEVICE = -4
ERR_ALLOC = -5
ERR_CAPACITY = -6
ERR_INTERNAL = -7
ERR_NAMES = {0: "OK", -1: "INVALID_ARG", -2: "CUDA", -3: "STEP_LIMIT", -4: "NO_DEVICE",
             -5: "ALLOC", -6: "CAPACITY", -7: "INTERNAL"}

MODE_COMPAT = 0
MODE_PHYSICAL = 1

# tally order = the reference's return order (ISMC.py:406)
TALLIES = ("A", "R_d", "R_s", "T_d", "T_u")


class Stack(C.Structure):
    _fields_ = [("L", C.c_uint32), ("_pad0", C.c_uint32),
                ("n", C.c_float * MAXL), ("mua", C.c_float * MAXL), ("mus", C.c_float * MAXL),
                ("mut", C.c_float * MAXL), ("g", C.c_float * MAXL), ("d", C.c_float * MAXL)]


class Spheres(C.Structure):
    _fields_ = [("R", C.c_uint8), ("T", C.c_uint8), ("specular_included", C.c_uint8),
                ("_pad0", C.c_uint8 * 5),
                ("R_pw", C.c_double), ("R_fs", C.c_double), ("R_fp", C.c_double),
                ("R_fd", C.c_double), ("R_f", C.c_double), ("R_angle", C.c_double),
                ("T_pw", C.c_double), ("T_fs", C.c_double), ("T_fp", C.c_double),
                ("T_fd", C.c_double), ("T_f", C.c_double), ("T_angle", C.c_double)]


class Instance(C.Structure):
    _fields_ = [("stack", Stack), ("spheres", Spheres), ("n_packets", C.c_uint64),
                ("packet_offset", C.c_uint64), ("seed", C.c_uint64), ("stream", C.c_uint32),
                ("mode", C.c_uint32), ("roulette_threshold", C.c_float),
                ("roulette_m", C.c_float)]


class Tally(C.Structure):
    _fields_ = [("n", C.c_uint64), ("sum", C.c_uint64 * 5), ("sumsq", C.c_uint64 * 5),
                ("steps", C.c_uint64), ("events", C.c_uint64), ("reincidences", C.c_uint64),
                ("capped", C.c_uint64), ("trapped", C.c_uint64), ("scale_log2", C.c_uint32), ("status", C.c_int32),
                ("analytic_specular", C.c_float), ("analytic_ballistic", C.c_float)]


class Tune(C.Structure):
    _fields_ = [("block_threads", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("chunk_packets", C.c_uint32), ("max_events", C.c_uint32)]


class SolveReq(C.Structure):
    _fields_ = [("base", Instance), ("layer", C.c_uint32), ("separate", C.c_uint32),
                ("log_coords", C.c_uint32), ("max_evals", C.c_uint32),
                ("max_restarts", C.c_uint32), ("fresh_streams", C.c_uint32),
                ("max_refits", C.c_uint32), ("_pad0", C.c_uint32),
                ("meas", C.c_double * 4), ("x0", C.c_double * 2), ("lo", C.c_double * 2),
                ("hi", C.c_double * 2), ("h0", C.c_double), ("t0", C.c_double)]


class SolveOut(C.Structure):
    _fields_ = [("x", C.c_double * 2), ("cost", C.c_double), ("evals", C.c_uint32),
                ("restarts", C.c_uint32), ("status", C.c_int32), ("rounds", C.c_uint32),
                ("refits", C.c_uint32), ("_pad0", C.c_uint32)]


OBJECTIVE = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_int, C.c_void_p)

SIZEOF_INDEX = {0: Stack, 1: Spheres, 2: Instance, 3: Tally, 4: Tune, 5: SolveReq, 6: SolveOut}

# every symbol include/ismc.h declares
EXPORTS = ("ismc_version", "ismc_init", "ismc_destroy", "ismc_run", "ismc_run_batch",
           "ismc_run_batch_device", "ismc_autotune", "ismc_last_error", "ismc_sizeof",
           "ismc_solve_batch", "ismc_praxis", "ismc_run_batch_noalloc", "ismc_validate",
           "ismc_mlp_create", "ismc_mlp_destroy", "ismc_mlp_nparam", "ismc_mlp_get_params",
           "ismc_mlp_set_params", "ismc_mlp_forward", "ismc_mlp_grad", "ismc_mlp_train_step",
           "ismc_mlp_sync", "ismc_mlp_gemm_test", "ismc_mlp_last_error", "ismc_mlp_train_epoch",
           "ismc_mlp_set_wait_limit",
           "ismc_table_interp", "ismc_table_interp_cubic", "ismc_table_uncertainty",
           "ismc_table_lookup")

NOALLOC_MAX_INST = 1024          # ISMC_NOALLOC_MAX_INST
MAX_PACKETS = 1 << 31            # ISMC_MAX_PACKETS: packets of one instance


def declare(lib):
    """Attach argtypes/restype to the library's entry points."""
    P = C.POINTER
    lib.ismc_version.restype = C.c_int
    lib.ismc_version.argtypes = []
    lib.ismc_init.restype = C.c_int
    lib.ismc_init.argtypes = [C.c_int, P(C.c_void_p)]
    lib.ismc_destroy.restype = C.c_int
    lib.ismc_destroy.argtypes = [C.c_void_p]
    lib.ismc_run.restype = C.c_int
    lib.ismc_run.argtypes = [C.c_void_p, P(Stack), P(Spheres), C.c_uint64, C.c_uint64, C.c_uint32,
                             P(Tally)]
    lib.ismc_run_batch.restype = C.c_int
    lib.ismc_run_batch.argtypes = [C.c_void_p, P(Instance), C.c_uint32, P(Tune), P(Tally)]
    lib.ismc_run_batch_device.restype = C.c_int
    lib.ismc_run_batch_device.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, P(Tune), C.c_void_p,
                                          C.c_void_p]
    lib.ismc_autotune.restype = C.c_int
    lib.ismc_autotune.argtypes = [C.c_void_p, P(Instance), C.c_uint32, P(Tune)]
    lib.ismc_last_error.restype = C.c_int
    lib.ismc_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    lib.ismc_solve_batch.restype = C.c_int
    lib.ismc_solve_batch.argtypes = [C.c_void_p, P(SolveReq), C.c_uint32, P(SolveOut)]
    lib.ismc_praxis.restype = C.c_int
    lib.ismc_praxis.argtypes = [OBJECTIVE, C.c_void_p, C.c_int, P(C.c_double), C.c_double,
                                C.c_double, C.c_int, P(C.c_double), P(C.c_int)]
    lib.ismc_validate.restype = C.c_int
    lib.ismc_validate.argtypes = [P(Instance), C.c_uint32, P(C.c_int32)]
    lib.ismc_run_batch_noalloc.restype = C.c_int
    lib.ismc_run_batch_noalloc.argtypes = [C.c_void_p, C.c_uint32, P(Tune), C.c_void_p, C.c_void_p]
    V, F = C.c_void_p, P(C.c_float)
    lib.ismc_mlp_create.restype = C.c_int
    lib.ismc_mlp_create.argtypes = [C.c_int, C.c_uint32, C.c_uint64, P(V)]
    lib.ismc_mlp_destroy.restype = C.c_int
    lib.ismc_mlp_destroy.argtypes = [V]
    lib.ismc_mlp_nparam.restype = C.c_size_t
    lib.ismc_mlp_nparam.argtypes = []
    lib.ismc_mlp_get_params.restype = C.c_int
    lib.ismc_mlp_get_params.argtypes = [V, F, C.c_size_t]
    lib.ismc_mlp_set_params.restype = C.c_int
    lib.ismc_mlp_set_params.argtypes = [V, F, C.c_size_t]
    lib.ismc_mlp_forward.restype = C.c_int
    lib.ismc_mlp_forward.argtypes = [V, V, C.c_uint32, V]
    lib.ismc_mlp_grad.restype = C.c_int
    lib.ismc_mlp_grad.argtypes = [V, V, V, C.c_uint32, V, F]
    lib.ismc_mlp_train_step.restype = C.c_int
    lib.ismc_mlp_train_step.argtypes = [V, V, V, C.c_uint32, C.c_float, F]
    lib.ismc_mlp_train_epoch.restype = C.c_int
    lib.ismc_mlp_train_epoch.argtypes = [V, V, V, C.c_uint32, C.c_uint32, F, F]
    lib.ismc_mlp_sync.restype = C.c_int
    lib.ismc_mlp_sync.argtypes = [V]
    lib.ismc_mlp_gemm_test.restype = C.c_int
    lib.ismc_mlp_gemm_test.argtypes = [V, V, V, V, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.ismc_mlp_set_wait_limit.restype = C.c_int
    lib.ismc_mlp_set_wait_limit.argtypes = [V, C.c_uint32]
    lib.ismc_mlp_last_error.restype = C.c_int
    lib.ismc_mlp_last_error.argtypes = [V, C.c_char_p, C.c_size_t]
    D = P(C.c_double)
    lib.ismc_table_interp.restype = C.c_int
    lib.ismc_table_interp.argtypes = [D, D, D, C.c_uint32, P(C.c_int32), C.c_uint32, C.c_uint32, D]
    lib.ismc_table_interp_cubic.restype = C.c_int
    lib.ismc_table_interp_cubic.argtypes = [D, D, D, C.c_uint32, P(C.c_int32), P(C.c_int32),
                                            C.c_uint32, P(C.c_int32), P(C.c_int32), C.c_uint32, D]
    lib.ismc_table_uncertainty.restype = C.c_int
    lib.ismc_table_uncertainty.argtypes = [D, D, D, D, C.c_uint32, C.c_uint32, C.c_uint64, D, D]
    lib.ismc_table_lookup.restype = C.c_int
    lib.ismc_table_lookup.argtypes = [D, C.c_uint32, D, D, C.c_uint32, D]
    lib.ismc_sizeof.restype = C.c_size_t
    lib.ismc_sizeof.argtypes = [C.c_int]
    for k, cls in SIZEOF_INDEX.items():
        got = lib.ismc_sizeof(k)
        if got != C.sizeof(cls):
            raise RuntimeError(f"ABI mismatch for {cls.__name__}: library {got} B, ctypes "
                               f"{C.sizeof(cls)} B")
    v = lib.ismc_version()
    if v != ABI_VERSION:
        raise RuntimeError(f"libismc ABI version {v}, bindings expect {ABI_VERSION}")
    return lib
