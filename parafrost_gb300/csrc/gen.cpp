// Seeded synthetic CNF families used as benchmark and test inputs.
//
// The reference ships no benchmark inputs; these generators produce the three
// instance families its simplifier is measured on (random k-SAT, Tseitin
// circuits, scale-free CNFs).  All arithmetic is integer (xoshiro256**), so x86
// and Arm hosts produce identical instances for the same seed.
//
// Output is the clause database the simplifier sees after the solver's own
// parse + root-level propagation (src/gpu/solver.cpp:46): unit clauses are
// propagated on the host, satisfied clauses dropped and false literals removed,
// so every emitted clause has >= 2 distinct literals in the internal encoding
// lit = 2*v | sign.
#include "pfgpu.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed + 0x9E3779B97F4A7C15ULL;
        for (int i = 0; i < 4; i++) {
            z += 0x9E3779B97F4A7C15ULL;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
            s[i] = x ^ (x >> 31);
        }
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    inline uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform in [0, n)
    inline uint64_t below(uint64_t n) {
        return (uint64_t)(((__uint128_t)next() * n) >> 64);
    }
    inline uint32_t bit() { return (uint32_t)(next() >> 63); }
    // uniform in [0,1) with 53 bits
    inline double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

struct Cnf {
    uint32_t maxVar = 0;
    std::vector<uint32_t> lits;
    std::vector<uint64_t> off{0};
    void add(const uint32_t* c, int n) {
        lits.insert(lits.end(), c, c + n);
        off.push_back(lits.size());
    }
};

inline uint32_t mklit(uint32_t v, uint32_t s) { return (v << 1) | s; }

// Root-level unit propagation over a clause list that may contain units.
// Returns false on conflict (the caller then keeps the unpropagated rest).
bool rootify(Cnf& in, Cnf& out) {
    const uint32_t V = in.maxVar;
    const size_t C = in.off.size() - 1;
    std::vector<int8_t> val(V + 1, 0);  // 0 unassigned, 1 true, -1 false
    std::vector<std::vector<uint32_t>> occ(2 * (size_t)V + 2);
    std::vector<uint32_t> queue;
    bool conflict = false;
    auto litval = [&](uint32_t l) -> int {
        int8_t x = val[l >> 1];
        return (l & 1) ? -x : x;
    };
    auto assign = [&](uint32_t l) {
        int cur = litval(l);
        if (cur == 1) return;
        if (cur == -1) { conflict = true; return; }
        val[l >> 1] = (l & 1) ? -1 : 1;
        queue.push_back(l);
    };
    for (size_t c = 0; c < C; c++) {
        const uint64_t b = in.off[c], e = in.off[c + 1];
        if (e - b == 1) assign(in.lits[b]);
        else for (uint64_t k = b; k < e; k++) occ[in.lits[k]].push_back((uint32_t)c);
    }
    for (size_t qi = 0; qi < queue.size() && !conflict; qi++) {
        const uint32_t f = queue[qi] ^ 1u;  // falsified literal
        for (uint32_t c : occ[f]) {
            const uint64_t b = in.off[c], e = in.off[c + 1];
            int unset = 0; uint32_t unit = 0; bool sat = false;
            for (uint64_t k = b; k < e; k++) {
                int lv = litval(in.lits[k]);
                if (lv == 1) { sat = true; break; }
                if (lv == 0) { unset++; unit = in.lits[k]; }
            }
            if (sat) continue;
            if (!unset) { conflict = true; break; }
            if (unset == 1) assign(unit);
        }
    }
    if (conflict) return false;
    out.maxVar = V;
    std::vector<uint32_t> tmp;
    for (size_t c = 0; c < C; c++) {
        const uint64_t b = in.off[c], e = in.off[c + 1];
        if (e - b == 1) continue;
        tmp.clear();
        bool sat = false;
        for (uint64_t k = b; k < e; k++) {
            int lv = litval(in.lits[k]);
            if (lv == 1) { sat = true; break; }
            if (lv == 0) tmp.push_back(in.lits[k]);
        }
        if (sat || tmp.size() < 2) continue;
        out.add(tmp.data(), (int)tmp.size());
    }
    return true;
}

void gen_ksat(uint32_t V, uint64_t C, int k, uint64_t seed, Cnf& out) {
    Rng r(seed);
    out.maxVar = V;
    out.lits.reserve(C * k);
    out.off.reserve(C + 1);
    uint32_t c[64];
    if (k > 64) k = 64;
    if ((uint32_t)k > V) k = (int)V;
    for (uint64_t i = 0; i < C; i++) {
        for (int j = 0; j < k; j++) {
            uint32_t v;
            bool dup;
            do {
                v = 1 + (uint32_t)r.below(V);
                dup = false;
                for (int t = 0; t < j; t++) if ((c[t] >> 1) == v) { dup = true; break; }
            } while (dup);
            c[j] = mklit(v, r.bit());
        }
        out.add(c, k);
    }
}

// Random 2-input circuit: nodes 1..P are primary inputs, node P+g is gate g
// (AND 40 %, OR 30 %, XOR 30 %) over two distinct earlier nodes; `outs`
// random gate outputs are asserted true and propagated at the root.
void gen_tseitin(uint64_t gates, uint64_t P, uint64_t outs, uint64_t seed, Cnf& out) {
    Rng r(seed);
    Cnf raw;
    const uint32_t V = (uint32_t)(P + gates);
    raw.maxVar = V;
    raw.lits.reserve(gates * 9);
    raw.off.reserve(gates * 34 / 10 + outs + 1);
    for (uint64_t g = 0; g < gates; g++) {
        const uint32_t node = (uint32_t)(P + g + 1);
        const uint32_t a = 1 + (uint32_t)r.below(node - 1);
        uint32_t b;
        do { b = 1 + (uint32_t)r.below(node - 1); } while (b == a);
        const uint64_t t = r.below(10);
        uint32_t c[3];
        if (t < 4) {  // AND: g = a & b
            c[0] = mklit(node, 1); c[1] = mklit(a, 0); raw.add(c, 2);
            c[0] = mklit(node, 1); c[1] = mklit(b, 0); raw.add(c, 2);
            c[0] = mklit(node, 0); c[1] = mklit(a, 1); c[2] = mklit(b, 1); raw.add(c, 3);
        } else if (t < 7) {  // OR: g = a | b
            c[0] = mklit(node, 0); c[1] = mklit(a, 1); raw.add(c, 2);
            c[0] = mklit(node, 0); c[1] = mklit(b, 1); raw.add(c, 2);
            c[0] = mklit(node, 1); c[1] = mklit(a, 0); c[2] = mklit(b, 0); raw.add(c, 3);
        } else {  // XOR: g = a ^ b
            c[0] = mklit(node, 1); c[1] = mklit(a, 0); c[2] = mklit(b, 0); raw.add(c, 3);
            c[0] = mklit(node, 1); c[1] = mklit(a, 1); c[2] = mklit(b, 1); raw.add(c, 3);
            c[0] = mklit(node, 0); c[1] = mklit(a, 1); c[2] = mklit(b, 0); raw.add(c, 3);
            c[0] = mklit(node, 0); c[1] = mklit(a, 0); c[2] = mklit(b, 1); raw.add(c, 3);
        }
    }
    for (uint64_t o = 0; o < outs && gates; o++) {
        const uint32_t node = (uint32_t)(P + 1 + r.below(gates));
        const uint32_t u = mklit(node, 0);
        raw.add(&u, 1);
    }
    if (!rootify(raw, out)) {
        // conflicting outputs: keep the circuit without the asserted outputs
        Cnf noouts;
        noouts.maxVar = V;
        for (size_t c = 0; c + 1 < raw.off.size(); c++) {
            const uint64_t b = raw.off[c], e = raw.off[c + 1];
            if (e - b >= 2) noouts.add(raw.lits.data() + b, (int)(e - b));
        }
        out = noouts;
    }
}

// Scale-free CNF: variable rank drawn with P(rank) ~ rank^(-1/(beta-1)),
// beta = 2.5, by the continuous inverse CDF rank = ceil(V * u^3); ranks are
// scattered over variable ids by an affine bijection; clause length is
// 2 + Geometric(p = 1/3) truncated to [2, 50] (mean ~4); distinct variables
// within a clause; random polarity. With `planted`, a hidden random
// assignment is drawn first and a clause that it falsifies gets the polarity
// of one random literal flipped, so the instance stays satisfiable.
void gen_scalefree(uint32_t V, uint64_t C, uint64_t seed, bool planted, Cnf& out) {
    Rng r(seed);
    std::vector<uint8_t> hidden;
    if (planted) {
        hidden.resize((size_t)V + 1);
        for (uint32_t v = 1; v <= V; v++) hidden[v] = (uint8_t)r.bit();
    }
    out.maxVar = V;
    out.lits.reserve(C * 4 + C / 8);
    out.off.reserve(C + 1);
    // affine bijection on [0, V): mult coprime with V
    uint64_t mult = 2654435761ULL % V;
    if (mult == 0) mult = 1;
    auto gcd = [](uint64_t a, uint64_t b) { while (b) { uint64_t t = a % b; a = b; b = t; } return a; };
    while (gcd(mult, V) != 1) mult++;
    const uint64_t add = (seed * 0x9E3779B97F4A7C15ULL) % V;
    uint32_t c[50];
    for (uint64_t i = 0; i < C; i++) {
        int len;
        do {
            len = 2;
            while (r.below(3) != 0) len++;  // geometric tail, success prob 1/3
        } while (len > 50);
        if ((uint32_t)len > V) len = (int)V;
        for (int j = 0; j < len; j++) {
            uint32_t v;
            bool dup;
            do {
                const double u = r.unit();
                uint64_t rank = (uint64_t)((double)V * u * u * u);
                if (rank >= V) rank = V - 1;
                v = 1 + (uint32_t)((rank * mult + add) % V);
                dup = false;
                for (int t = 0; t < j; t++) if ((c[t] >> 1) == v) { dup = true; break; }
            } while (dup);
            c[j] = mklit(v, r.bit());
        }
        if (planted) {
            bool sat = false;
            for (int j = 0; j < len && !sat; j++) sat = ((c[j] & 1u) ^ 1u) == hidden[c[j] >> 1];
            if (!sat) {
                const int j = (int)r.below((uint64_t)len);
                c[j] ^= 1u;
            }
        }
        out.add(c, len);
    }
}

}  // namespace

extern "C" int pfg_generate(int family, uint64_t a, uint64_t b, uint64_t c, uint64_t seed,
                            uint32_t* max_var, uint64_t* num_clauses, uint64_t* num_lits,
                            uint32_t* lits, uint64_t* cls_off) {
    // The generator is deterministic, so the sizing call and the filling call
    // produce the same instance; the last instance is kept per thread so the
    // filling call does not generate it twice.
    thread_local Cnf cached;
    thread_local uint64_t key[5] = {~0ULL, 0, 0, 0, 0};
    const uint64_t want[5] = {(uint64_t)family, a, b, c, seed};
    if (std::memcmp(key, want, sizeof(want)) != 0) {
        Cnf cnf;
        switch (family) {
            case 0:
                if (!a || a > 0x7FFFFFFEULL || c < 2) return PFG_INVALID;
                gen_ksat((uint32_t)a, b, (int)c, seed, cnf);
                break;
            case 1:
                if (b < 2 || a + b > 0x7FFFFFFEULL) return PFG_INVALID;
                gen_tseitin(a, b, c, seed, cnf);
                break;
            case 2:
                if (a < 2 || a > 0x7FFFFFFEULL) return PFG_INVALID;
                gen_scalefree((uint32_t)a, b, seed, c != 0, cnf);
                break;
            default:
                return PFG_INVALID;
        }
        cached = std::move(cnf);
        std::memcpy(key, want, sizeof(want));
    }
    const Cnf& cnf = cached;
    if (max_var) *max_var = cnf.maxVar;
    if (num_clauses) *num_clauses = cnf.off.size() - 1;
    if (num_lits) *num_lits = cnf.lits.size();
    if (lits) std::memcpy(lits, cnf.lits.data(), cnf.lits.size() * sizeof(uint32_t));
    if (cls_off) std::memcpy(cls_off, cnf.off.data(), cnf.off.size() * sizeof(uint64_t));
    return PFG_OK;
}
