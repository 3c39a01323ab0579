"""ctypes mirrors of the structs declared in include/pfgpu.h."""
import ctypes as C

PFG_OK = 0
PFG_AWAKEN_FAIL = 1
PFG_CNFALLOC_FAIL = 2
PFG_OTALLOC_FAIL = 3
PFG_TIMEOUT = 4
PFG_INVALID = 5
PFG_CUDA_ERROR = 6

PFG_UNKNOWN = 0
PFG_SAT = 10
PFG_UNSAT = 20

RETURN_NAMES = {
    PFG_OK: "ok",
    PFG_AWAKEN_FAIL: "awaken failed",
    PFG_CNFALLOC_FAIL: "CNF allocation failed",
    PFG_OTALLOC_FAIL: "occurrence table allocation failed",
    PFG_TIMEOUT: "device-side loop timed out",
    PFG_INVALID: "invalid input",
    PFG_CUDA_ERROR: "CUDA error",
    7: "job pending",
}


class PfgOptions(C.Structure):
    _fields_ = [
        ("phases", C.c_int32),
        ("shrink_rate", C.c_int32),
        ("lcve_fast", C.c_int32),
        ("lcve_min_vars", C.c_uint32),
        ("lcve_max_occurs", C.c_uint32),
        ("lcve_clause_max", C.c_int32),
        ("phase_lits_min", C.c_uint32),
        ("mu_pos", C.c_uint32),
        ("mu_neg", C.c_uint32),
        ("lits_mul", C.c_double),
        ("ve_en", C.c_uint8),
        ("ve_plus_en", C.c_uint8),
        ("sub_en", C.c_uint8),
        ("ere_en", C.c_uint8),
        ("bce_en", C.c_uint8),
        ("all_en", C.c_uint8),
        ("ve_fun_en", C.c_uint8),
        ("ve_lbound_en", C.c_uint8),
        ("proof_en", C.c_uint8),
        ("ve_inprocess", C.c_uint8),
        ("_pad", C.c_uint8 * 6),
        ("ve_clause_max", C.c_uint32),
        ("xor_max_arity", C.c_uint32),
        ("sub_max_occurs", C.c_uint32),
        ("ere_max_occurs", C.c_uint32),
        ("ere_clause_max", C.c_uint32),
        ("bce_max_occurs", C.c_uint32),
    ]


class PfgStats(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("rounds", C.c_int32),
        ("ere_ran", C.c_int32),
        ("simpstate", C.c_int32),
        ("clauses_in", C.c_uint64),
        ("literals_in", C.c_uint64),
        ("clauses_out", C.c_uint64),
        ("literals_out", C.c_uint64),
        ("clauses_processed", C.c_uint64),
        ("literals_processed", C.c_uint64),
        ("eliminated", C.c_uint64),
        ("forced", C.c_uint64),
        ("resolvents", C.c_uint64),
        ("stack_words", C.c_uint64),
        ("device_ms", C.c_double),
        ("pass_ms", C.c_double * 8),
        ("alg_bytes", C.c_uint64),
        ("kernel_launches", C.c_uint64),
    ]


class PfgResultSizes(C.Structure):
    _fields_ = [
        ("clauses", C.c_uint64),
        ("literals", C.c_uint64),
        ("units", C.c_uint64),
        ("pending_units", C.c_uint64),
        ("stack_words", C.c_uint64),
        ("rounds", C.c_uint64),
        ("max_var", C.c_uint32),
        ("_pad", C.c_uint32),
        ("proof_bytes", C.c_uint64),
    ]


class PfgInstance(C.Structure):
    """One instance of a batch (pfg_instance). The array pointers are plain
    addresses (c_void_p, the same layout as the typed pointers of the header):
    a host filling hundreds of these per call assigns integers instead of
    building ctypes pointer objects."""
    _fields_ = [
        ("max_var", C.c_uint32),
        ("_pad", C.c_uint32),
        ("num_clauses", C.c_uint64),
        ("lits", C.c_void_p),          # const uint32_t*
        ("cls_off", C.c_void_p),       # const uint64_t*
        ("cls_learnt", C.c_void_p),    # const uint8_t*
        ("cls_lbd", C.c_void_p),       # const uint32_t*
        ("cls_usage", C.c_void_p),     # const uint8_t*
        ("var_state", C.c_void_p),     # const uint8_t*
        ("assumed", C.c_void_p),       # const uint8_t*
        ("vorg", C.c_void_p),          # const uint32_t*
    ]


class PfgJobInfo(C.Structure):
    """Serving: state of one finished job (pfg_job_info)."""
    _fields_ = [
        ("rc", C.c_int32),
        ("status", C.c_int32),
        ("batch_size", C.c_uint32),
        ("slot", C.c_uint32),
        ("est_bytes", C.c_uint64),
        ("t_submit_ns", C.c_uint64),
        ("t_admit_ns", C.c_uint64),
        ("t_done_ns", C.c_uint64),
        ("clauses_processed", C.c_uint64),
        ("sizes", PfgResultSizes),
    ]


class PfgServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_uint64),
        ("admitted", C.c_uint64),
        ("done", C.c_uint64),
        ("batches", C.c_uint64),
        ("max_in_flight_batches", C.c_uint64),
        ("max_jobs_in_flight", C.c_uint64),
        ("peak_est_bytes", C.c_uint64),
        ("budget_bytes", C.c_uint64),
    ]


class PfgDimacsInfo(C.Structure):
    _fields_ = [
        ("max_var", C.c_uint32),
        ("status", C.c_int32),
        ("header_clauses", C.c_uint64),
        ("num_clauses", C.c_uint64),
        ("num_literals", C.c_uint64),
        ("num_units", C.c_uint64),
    ]


class PfgTuning(C.Structure):
    """pfg_tuning: launch shapes per pass (0 = the built-in choice)."""
    _fields_ = [
        ("sub_blocks_per_sm", C.c_uint32),
        ("ve1_blocks_per_sm", C.c_uint32),
        ("ve3_blocks_per_sm", C.c_uint32),
        ("ve3_ticket", C.c_uint32),
        ("mis_threads", C.c_uint32),
        ("list_threads", C.c_uint32),
        ("bcp_blocks_per_sm", C.c_uint32),
        ("_reserved", C.c_uint32 * 9),
    ]


PFG_PENDING = 7

PASS_NAMES = ("ot", "bcp", "lcve", "sub", "ve", "ere", "gc", "other")

# Reference option names (src/gpu/options.cpp:24-43, options.cu:33-60) -> struct fields.
CLI_NAMES = {
    "phases": "phases",
    "collectfreq": "shrink_rate",
    "lcvefast": "lcve_fast",
    "electionsmin": "lcve_min_vars",
    "electionsmax": "lcve_max_occurs",
    "lcveclausemax": "lcve_clause_max",
    "eliminatedlitsmin": "phase_lits_min",
    "mupos": "mu_pos",
    "muneg": "mu_neg",
    "literalsmul": "lits_mul",
    "ve": "ve_en",
    "veextend": "ve_plus_en",
    "sub": "sub_en",
    "ere": "ere_en",
    "bce": "bce_en",
    "all": "all_en",
    "vefunction": "ve_fun_en",
    "velitsbound": "ve_lbound_en",
    "proof": "proof_en",
    "resolventmax": "ve_clause_max",
    "xormaxarity": "xor_max_arity",
    "submaxoccurs": "sub_max_occurs",
    "eremaxoccurs": "ere_max_occurs",
    "ereclausemax": "ere_clause_max",
    "bcemaxoccurs": "bce_max_occurs",
}


def default_options() -> PfgOptions:
    """Reference defaults (options.cpp:24-43, options.cu:33-60)."""
    o = PfgOptions()
    o.phases = 5
    o.shrink_rate = 2
    o.lcve_fast = 1
    o.lcve_min_vars = 2
    o.lcve_max_occurs = 3000
    o.lcve_clause_max = 30000
    o.phase_lits_min = 500
    o.mu_pos = 32
    o.mu_neg = 32
    o.lits_mul = 1.0
    o.ve_en = 1
    o.ve_plus_en = 1
    o.sub_en = 1
    o.ere_en = 1
    o.bce_en = 0
    o.all_en = 0
    o.ve_fun_en = 1
    o.ve_lbound_en = 0
    o.proof_en = 0
    o.ve_inprocess = 0
    o.ve_clause_max = 100
    o.xor_max_arity = 10
    o.sub_max_occurs = 3000
    o.ere_max_occurs = 3000
    o.ere_clause_max = 250
    o.bce_max_occurs = 3000
    return o


def options_from(**kw) -> PfgOptions:
    """Options from reference CLI names (`phases=1, ere=False`) or struct field names."""
    o = default_options()
    for k, v in kw.items():
        field = CLI_NAMES.get(k, k)
        if not any(f[0] == field for f in PfgOptions._fields_):
            raise KeyError(f"unknown simplifier option {k!r}")
        if isinstance(v, bool):
            v = int(v)
        setattr(o, field, v)
    return o


def options_dict(o: PfgOptions) -> dict:
    return {f[0]: getattr(o, f[0]) for f in PfgOptions._fields_ if not f[0].startswith("_")}
