// Write-back helpers for the host solver: variable compaction after
// simplification and model reconstruction from the model stack.
//
// pfg_map_vars follows VMAP::initiate / mapLit (src/gpu/vmap.hpp:44-72): the
// variables still active (eliminated byte 0: neither eliminated nor fixed by
// propagation) keep their relative order and are renumbered 1..n; eliminated
// and fixed variables get no new number. pfg_extend_model follows
// MODEL::extend (src/gpu/model.cpp:101-160): the stack is walked from the end;
// a saved clause that the current values falsify makes its first (witness)
// literal true.
#include <cstdint>

#include "pfgpu.h"

extern "C" int pfg_map_vars(uint32_t max_var, const uint8_t* eliminated, uint32_t* new_of_old, uint32_t* old_of_new,
                            uint32_t* new_max_var) {
    if (!eliminated || !new_of_old || !new_max_var) return PFG_INVALID;
    uint32_t n = 0;
    new_of_old[0] = 0;
    if (old_of_new) old_of_new[0] = 0;
    for (uint32_t v = 1; v <= max_var; v++) {
        if (eliminated[v]) { new_of_old[v] = 0; continue; }
        new_of_old[v] = ++n;
        if (old_of_new) old_of_new[n] = v;
    }
    *new_max_var = n;
    return PFG_OK;
}

extern "C" int pfg_map_lits(const uint32_t* new_of_old, uint32_t max_var, uint64_t n, const uint32_t* in,
                            uint32_t* out) {
    if (!new_of_old || (n && (!in || !out))) return PFG_INVALID;
    for (uint64_t i = 0; i < n; i++) {
        const uint32_t v = in[i] >> 1;
        if (v == 0 || v > max_var || !new_of_old[v]) return PFG_INVALID;   // literal of a dropped variable
        out[i] = (new_of_old[v] << 1) | (in[i] & 1u);
    }
    return PFG_OK;
}

// value[v] for v in 1..max_var: 0 false, 1 true (every variable set on entry)
extern "C" int pfg_extend_model(uint64_t nstack, const uint32_t* stack, uint32_t max_var, uint8_t* value) {
    if (!value || (nstack && !stack)) return PFG_INVALID;
    uint64_t x = nstack;
    while (x > 0) {
        const uint32_t k = stack[x - 1];
        if (k == 0 || k > x - 1) return PFG_INVALID;              // malformed stack
        const uint64_t b = x - 1 - k;                              // clause stack[b .. b+k)
        bool sat = false;
        for (uint64_t i = b + 1; i < x - 1 && !sat; i++) {
            const uint32_t l = stack[i], v = l >> 1;
            if (v == 0 || v > max_var) return PFG_INVALID;
            sat = value[v] != (l & 1u);
        }
        const uint32_t w = stack[b], wv = w >> 1;
        if (wv == 0 || wv > max_var) return PFG_INVALID;
        if (!sat && value[wv] == (w & 1u)) value[wv] = (uint8_t)((w & 1u) ^ 1u);   // the witness becomes true
        x = b;
    }
    return PFG_OK;
}
