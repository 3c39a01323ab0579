// Text form of a binary DRAT proof, as the reference writes a proof file
// when binary output is off (cuPROOF::writeClause / writeProof,
// src/gpu/proof.cu:130-180): "d " before a deletion, every literal as a
// signed decimal variable followed by a space, then "0\n".
#include <cstdint>
#include <cstring>

#include "pfgpu.h"

namespace {

struct Sink {
    char* out;
    uint64_t cap, n;
    void put(char ch) {
        if (out && n < cap) out[n] = ch;
        n++;
    }
};

}  // namespace

extern "C" int pfg_proof_text(const uint8_t* bin, uint64_t n, char* out, uint64_t cap, uint64_t* len) {
    if (!len || (n && !bin)) return PFG_INVALID;
    Sink s{out, cap, 0};
    uint64_t p = 0;
    while (p < n) {
        const uint8_t state = bin[p++];
        if (state != 97u && state != 100u) return PFG_INVALID;
        if (state == 100u) { s.put('d'); s.put(' '); }
        while (true) {
            if (p >= n) return PFG_INVALID;          // no terminator
            if (bin[p] == 0) { p++; break; }
            uint64_t v = 0;
            uint32_t shift = 0;
            uint8_t b;
            do {
                if (p >= n || shift > 28) return PFG_INVALID;
                b = bin[p++];
                v |= (uint64_t)(b & 0x7Fu) << shift;
                shift += 7;
            } while (b & 0x80u);
            if (v < 2) return PFG_INVALID;
            if (v & 1u) s.put('-');
            char digits[24];
            int k = 0;
            for (uint64_t d = v >> 1; d; d /= 10) digits[k++] = (char)('0' + d % 10);
            while (k) s.put(digits[--k]);
            s.put(' ');
        }
        s.put('0');
        s.put('\n');
    }
    *len = s.n;
    return PFG_OK;
}
