// DIMACS CNF ingest feeding pfg_upload / pfg_batch_upload directly.
//
// Follows Solver::parse / toClause (src/gpu/dimacs.cpp:41-290): the file is
// memory-mapped; "c" lines are comments; the "p cnf V C" header fixes the
// variable range; in every clause repeated literals are dropped, a clause with
// a literal and its negation is dropped (satisfied), literals of units read
// earlier in the file are applied (a true literal drops the clause, a false one
// is removed), a clause left with one literal becomes a unit (or a conflict),
// and an empty clause makes the formula UNSAT. Clauses keep their literal
// order; literals use the engine's encoding 2v|s.
#include <cerrno>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "pfgpu.h"

struct pfg_dimacs {
    pfg_dimacs_info info{};
    std::vector<uint32_t> lits;
    std::vector<uint64_t> off;
    std::vector<uint32_t> units;
    std::string err;
};

namespace {

struct Reader {
    const char* p;
    const char* end;
    bool eof() const { return p >= end; }
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
    }
    void line() {
        while (p < end && *p != '\n') p++;
        if (p < end) p++;
    }
    // signed decimal; false when no digits follow
    bool integer(int64_t& out) {
        ws();
        bool neg = false;
        if (p < end && (*p == '-' || *p == '+')) { neg = *p == '-'; p++; }
        if (p >= end || *p < '0' || *p > '9') return false;
        int64_t v = 0;
        while (p < end && *p >= '0' && *p <= '9') {
            v = v * 10 + (*p - '0');
            if (v > (int64_t)1 << 40) return false;
            p++;
        }
        out = neg ? -v : v;
        return true;
    }
};

bool parse(pfg_dimacs& d, const char* buf, size_t n) {
    Reader r{buf, buf + n};
    bool header = false;
    uint32_t V = 0;
    std::vector<uint8_t> mark;    // per literal: seen in the current clause
    std::vector<int8_t> value;    // per variable: 0 unassigned, 1 true, -1 false (units read so far)
    std::vector<uint32_t> cls, org;
    d.off.push_back(0);
    while (true) {
        r.ws();
        if (r.eof() || *r.p == '%') break;
        if (*r.p == 'c') { r.line(); continue; }
        if (*r.p == 'p') {
            if (header) { d.err = "second header"; return false; }
            if ((size_t)(r.end - r.p) < 5 || std::strncmp(r.p, "p cnf", 5) != 0) { d.err = "header has wrong format"; return false; }
            r.p += 5;
            int64_t nv = 0, nc = 0;
            if (!r.integer(nv) || !r.integer(nc)) { d.err = "header has wrong format"; return false; }
            if (nv <= 0) { d.err = "zero or negative number of variables in header"; return false; }
            if (nv >= 0x7FFFFFF0ll) { d.err = "number of variables not supported"; return false; }
            if (nc <= 0) { d.err = "zero or negative number of clauses in header"; return false; }
            V = (uint32_t)nv;
            d.info.max_var = V;
            d.info.header_clauses = (uint64_t)nc;
            mark.assign(2ull * V + 2, 0);
            value.assign((size_t)V + 1, 0);
            header = true;
            continue;
        }
        if (!header) { d.err = "expected 'c' or 'p' before the first clause"; return false; }
        // one clause, terminated by 0
        cls.clear();
        org.clear();
        bool satisfied = false;
        while (true) {
            int64_t x = 0;
            if (!r.integer(x)) { d.err = "unterminated clause or bad literal"; return false; }
            if (x == 0) break;
            const uint64_t v = (uint64_t)(x < 0 ? -x : x);
            if (v > V) { d.err = "too many variables"; return false; }
            const uint32_t lit = (uint32_t)(2 * v + (x < 0 ? 1 : 0));
            org.push_back(lit);
            if (mark[lit]) continue;                       // repeated literal
            if (mark[lit ^ 1u]) { satisfied = true; continue; }   // tautology
            mark[lit] = 1;
            const int8_t val = value[v];
            if (!val) cls.push_back(lit);
            else if ((val > 0) == !(lit & 1u)) satisfied = true;  // true literal
        }
        for (uint32_t l : org) mark[l] = 0;
        if (satisfied) continue;
        if (cls.empty()) {                                   // empty clause
            d.info.status = PFG_UNSAT;
            return true;
        }
        if (cls.size() == 1) {
            const uint32_t u = cls[0], v = u >> 1;
            if (!value[v]) {
                value[v] = (u & 1u) ? -1 : 1;
                d.units.push_back(u);
            }
            continue;
        }
        d.lits.insert(d.lits.end(), cls.begin(), cls.end());
        d.off.push_back(d.lits.size());
    }
    if (!header) { d.err = "no header"; return false; }
    return true;
}

}  // namespace

extern "C" int pfg_dimacs_read(const char* path, pfg_dimacs** out) {
    if (!out) return PFG_INVALID;
    pfg_dimacs* d = new pfg_dimacs();
    *out = d;
    if (!path) { d->err = "no path"; return PFG_INVALID; }
    const int fd = open(path, O_RDONLY);
    if (fd < 0) { d->err = std::string("cannot open input file: ") + std::strerror(errno); return PFG_INVALID; }
    struct stat st;
    if (fstat(fd, &st) != 0) { close(fd); d->err = "cannot stat input file"; return PFG_INVALID; }
    bool ok = true;
    if (st.st_size > 0) {
        void* m = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
        if (m == MAP_FAILED) { close(fd); d->err = "cannot map input file"; return PFG_INVALID; }
        ok = parse(*d, (const char*)m, (size_t)st.st_size);
        munmap(m, (size_t)st.st_size);
    } else {
        d->err = "empty input file";
        ok = false;
    }
    close(fd);
    if (!ok) return PFG_INVALID;
    d->info.num_clauses = d->off.size() - 1;
    d->info.num_literals = d->lits.size();
    d->info.num_units = d->units.size();
    return PFG_OK;
}

extern "C" int pfg_dimacs_get_info(pfg_dimacs* d, pfg_dimacs_info* info) {
    if (!d || !info) return PFG_INVALID;
    *info = d->info;
    return PFG_OK;
}

extern "C" int pfg_dimacs_copy(pfg_dimacs* d, uint32_t* lits, uint64_t* cls_off, uint32_t* units) {
    if (!d) return PFG_INVALID;
    if (lits && !d->lits.empty()) std::memcpy(lits, d->lits.data(), d->lits.size() * sizeof(uint32_t));
    if (cls_off) std::memcpy(cls_off, d->off.data(), d->off.size() * sizeof(uint64_t));
    if (units && !d->units.empty()) std::memcpy(units, d->units.data(), d->units.size() * sizeof(uint32_t));
    return PFG_OK;
}

extern "C" const char* pfg_dimacs_error(pfg_dimacs* d) { return d ? d->err.c_str() : "null handle"; }

extern "C" void pfg_dimacs_free(pfg_dimacs* d) { delete d; }
