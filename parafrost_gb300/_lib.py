"""Loader of the engine library `libpfgpu.so` (ctypes, C ABI of include/pfgpu.h).

The library is built in-tree by `parafrost_gb300.build`; there is no other
implementation to fall back to, so a missing or broken library raises.
"""
import ctypes as C
import os

from ._abi import (PfgDimacsInfo, PfgInstance, PfgJobInfo, PfgOptions, PfgResultSizes, PfgServerStats, PfgStats,
                   PfgTuning)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpfgpu.so")
GEN_LIB_PATH = os.path.join(_HERE, "libpfgen.so")
_lib = None
_gen = None

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build the CUDA engine first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(LIB_PATH)
    L.pfg_abi_sizes.argtypes = [C.POINTER(C.c_size_t)] * 3
    L.pfg_abi_sizes.restype = None
    L.pfg_default_options.argtypes = [C.POINTER(PfgOptions)]
    L.pfg_default_options.restype = None
    L.pfg_resolve_options.argtypes = [C.POINTER(PfgOptions)]
    L.pfg_resolve_options.restype = None
    L.pfg_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(PfgOptions), C.c_size_t]
    L.pfg_create.restype = C.c_int
    L.pfg_upload.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, u32p, u64p, u8p, u32p, u8p, u8p, u8p, u32p]
    L.pfg_upload.restype = C.c_int
    L.pfg_simplify.argtypes = [C.c_void_p, C.POINTER(PfgStats)]
    L.pfg_simplify.restype = C.c_int
    L.pfg_simplify_many.argtypes = [C.POINTER(C.c_void_p), C.c_uint32, C.POINTER(PfgStats), C.POINTER(C.c_float)]
    L.pfg_simplify_many.restype = C.c_int
    L.pfg_result_sizes_get.argtypes = [C.c_void_p, C.POINTER(PfgResultSizes)]
    L.pfg_result_sizes_get.restype = C.c_int
    L.pfg_download.argtypes = [C.c_void_p, u32p, u64p, u8p, u32p, u8p, u8p, u32p, u32p, u32p, u64p]
    L.pfg_download.restype = C.c_int
    L.pfg_batch_upload.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(PfgInstance)]
    L.pfg_batch_upload.restype = C.c_int
    L.pfg_batch_size.argtypes = [C.c_void_p]
    L.pfg_batch_size.restype = C.c_uint32
    L.pfg_batch_stats.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(PfgStats)]
    L.pfg_batch_stats.restype = C.c_int
    L.pfg_batch_result_sizes.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(PfgResultSizes)]
    L.pfg_batch_result_sizes.restype = C.c_int
    L.pfg_batch_download.argtypes = [C.c_void_p, C.c_uint32, u32p, u64p, u8p, u32p, u8p, u8p, u32p, u32p, u32p, u64p]
    L.pfg_batch_download.restype = C.c_int
    L.pfg_batch_result_sizes_all.argtypes = [C.c_void_p, C.POINTER(PfgResultSizes)]
    L.pfg_batch_result_sizes_all.restype = C.c_int
    L.pfg_batch_download_all.argtypes = [C.c_void_p, u32p, u64p, u8p, u32p, u8p, u8p, u32p, u32p, u32p, u64p]
    L.pfg_batch_download_all.restype = C.c_int
    L.pfg_download_device_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.pfg_download_device_noalloc.restype = C.c_int
    L.pfg_server_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(PfgOptions), C.c_size_t, C.c_uint32, C.c_uint32]
    L.pfg_server_create.restype = C.c_int
    L.pfg_server_submit.argtypes = [C.c_void_p, C.POINTER(PfgInstance), C.POINTER(C.c_uint64)]
    L.pfg_server_submit.restype = C.c_int
    L.pfg_server_poll.argtypes = [C.c_void_p, C.c_uint64, C.c_int32, C.POINTER(PfgJobInfo)]
    L.pfg_server_poll.restype = C.c_int
    L.pfg_server_fetch.argtypes = [C.c_void_p, C.c_uint64, u32p, u64p, u8p, u32p, u8p, u8p, u32p, u32p, u32p, u64p]
    L.pfg_server_fetch.restype = C.c_int
    L.pfg_server_stats_get.argtypes = [C.c_void_p, C.POINTER(PfgServerStats)]
    L.pfg_server_stats_get.restype = C.c_int
    L.pfg_server_destroy.argtypes = [C.c_void_p]
    L.pfg_server_destroy.restype = None
    L.pfg_server_last_error.argtypes = [C.c_void_p]
    L.pfg_server_last_error.restype = C.c_char_p
    L.pfg_dimacs_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    L.pfg_dimacs_read.restype = C.c_int
    L.pfg_dimacs_get_info.argtypes = [C.c_void_p, C.POINTER(PfgDimacsInfo)]
    L.pfg_dimacs_get_info.restype = C.c_int
    L.pfg_dimacs_copy.argtypes = [C.c_void_p, u32p, u64p, u32p]
    L.pfg_dimacs_copy.restype = C.c_int
    L.pfg_dimacs_error.argtypes = [C.c_void_p]
    L.pfg_dimacs_error.restype = C.c_char_p
    L.pfg_dimacs_free.argtypes = [C.c_void_p]
    L.pfg_dimacs_free.restype = None
    L.pfg_map_vars.argtypes = [C.c_uint32, u8p, u32p, u32p, C.POINTER(C.c_uint32)]
    L.pfg_map_vars.restype = C.c_int
    L.pfg_map_lits.argtypes = [u32p, C.c_uint32, C.c_uint64, u32p, u32p]
    L.pfg_map_lits.restype = C.c_int
    L.pfg_extend_model.argtypes = [C.c_uint64, u32p, C.c_uint32, u8p]
    L.pfg_extend_model.restype = C.c_int
    L.pfg_download_proof.argtypes = [C.c_void_p, u8p]
    L.pfg_download_proof.restype = C.c_int
    L.pfg_batch_download_proof.argtypes = [C.c_void_p, C.c_uint32, u8p]
    L.pfg_batch_download_proof.restype = C.c_int
    L.pfg_proof_text.argtypes = [u8p, C.c_uint64, C.c_char_p, C.c_uint64, u64p]
    L.pfg_proof_text.restype = C.c_int
    L.pfg_host_alloc.argtypes = [C.c_size_t]
    L.pfg_host_alloc.restype = C.c_void_p
    L.pfg_host_free.argtypes = [C.c_void_p]
    L.pfg_host_free.restype = None
    L.pfg_tuning_get.argtypes = [C.c_void_p, C.POINTER(PfgTuning)]
    L.pfg_tuning_get.restype = C.c_int
    L.pfg_set_loop_limits.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32]
    L.pfg_set_loop_limits.restype = C.c_int
    L.pfg_tuning_set.argtypes = [C.c_void_p, C.POINTER(PfgTuning)]
    L.pfg_tuning_set.restype = C.c_int
    L.pfg_autotune.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(PfgInstance), C.c_uint32, C.POINTER(PfgTuning)]
    L.pfg_autotune.restype = C.c_int
    L.pfg_server_fetch_proof.argtypes = [C.c_void_p, C.c_uint64, u8p]
    L.pfg_server_fetch_proof.restype = C.c_int
    L.pfg_destroy.argtypes = [C.c_void_p]
    L.pfg_destroy.restype = None
    L.pfg_last_error.argtypes = [C.c_void_p]
    L.pfg_last_error.restype = C.c_char_p
    L.pfg_kernel_launches.argtypes = [C.c_void_p]
    L.pfg_kernel_launches.restype = C.c_uint64
    L.pfg_profile_enable.argtypes = [C.c_void_p, C.c_int]
    L.pfg_profile_enable.restype = C.c_int
    L.pfg_profile_reset.argtypes = [C.c_void_p]
    L.pfg_profile_reset.restype = None
    L.pfg_profile_count.argtypes = []
    L.pfg_profile_count.restype = C.c_int
    L.pfg_profile_name.argtypes = [C.c_int]
    L.pfg_profile_name.restype = C.c_char_p
    L.pfg_profile_get.argtypes = [C.c_void_p, C.c_int, u64p, C.POINTER(C.c_double), u64p]
    L.pfg_profile_get.restype = C.c_int
    L.pfg_generate.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                               u32p, u64p, u64p, u32p, u64p]
    L.pfg_generate.restype = C.c_int
    _lib = L
    return L


def gen_lib():
    """The host-only generator library (pfg_generate without the engine)."""
    global _gen
    if _gen is not None:
        return _gen
    if not os.path.exists(GEN_LIB_PATH):
        raise RuntimeError(
            f"{GEN_LIB_PATH} is missing: build first (python -c 'import __graft_entry__ as g; g.build()')")
    G = C.CDLL(GEN_LIB_PATH)
    G.pfg_generate.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                               u32p, u64p, u64p, u32p, u64p]
    G.pfg_generate.restype = C.c_int
    _gen = G
    return G


# C-ABI entry points declared in include/pfgpu.h (checked by the CPU tests)
EXPORTED = (
    "pfg_abi_sizes", "pfg_default_options", "pfg_resolve_options", "pfg_create", "pfg_upload", "pfg_simplify",
    "pfg_result_sizes_get", "pfg_download", "pfg_destroy", "pfg_last_error", "pfg_kernel_launches",
    "pfg_generate", "pfg_profile_enable", "pfg_profile_reset", "pfg_profile_count", "pfg_profile_name",
    "pfg_profile_get", "pfg_batch_upload", "pfg_batch_size", "pfg_batch_stats", "pfg_batch_result_sizes",
    "pfg_batch_download", "pfg_batch_result_sizes_all", "pfg_batch_download_all", "pfg_download_device_noalloc", "pfg_server_create", "pfg_server_submit",
    "pfg_server_poll", "pfg_server_fetch", "pfg_server_stats_get", "pfg_server_destroy", "pfg_server_last_error",
    "pfg_dimacs_read", "pfg_dimacs_get_info", "pfg_dimacs_copy", "pfg_dimacs_error", "pfg_dimacs_free",
    "pfg_map_vars", "pfg_map_lits", "pfg_extend_model", "pfg_download_proof", "pfg_batch_download_proof",
    "pfg_proof_text", "pfg_host_alloc", "pfg_host_free", "pfg_tuning_get", "pfg_tuning_set", "pfg_autotune",
    "pfg_set_loop_limits", "pfg_simplify_many",
    "pfg_server_fetch_proof",
)
