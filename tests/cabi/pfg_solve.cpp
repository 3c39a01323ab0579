/*
 * pfg_solve.cpp - a C++ host of the engine's C ABI (include/pfgpu.h), built
 * and run by tests/test_cabi.py.
 *
 * It is what a solver's simplify call site does with the library, end to
 * end: read a DIMACS file (pfg_dimacs_read), assign its unit clauses at the
 * root and drop what they satisfy (what the reference's parser and
 * rootify/shrinkTop leave for awaken, src/gpu/solver.cpp:42-48,
 * simplify.cu:143-145), simplify on the GPU (pfg_create, pfg_upload,
 * pfg_simplify, pfg_result_sizes_get, pfg_download, pfg_destroy), renumber
 * the active variables (pfg_map_vars/pfg_map_lits, as Solver::map,
 * src/gpu/vmap.cpp:61), hand the mapped formula to an external solver, and
 * take its model back to the original formula (pfg_extend_model, as
 * MODEL::extend, src/gpu/model.cpp:101-160), which is then checked against
 * every original clause. The same CNF also goes once through a two-instance
 * batch (pfg_batch_*), once into two contexts simplified at once
 * (pfg_simplify_many) and once through the serving loop (pfg_server_*); every
 * result must equal the single call's.
 *
 * usage: pfg_solve <in.cnf> <work-dir> [solver [solver options...]]
 * The simplify input and outputs are written to <work-dir>/simp.in and
 * simp.out (the layout tests/refgpu.py reads), the mapped formula to
 * <work-dir>/mapped.cnf. The solver is run as `solver mapped.cnf options`; it must
 * print "s SATISFIABLE" with "v" lines, or "s UNSATISFIABLE". Output: lines
 * "result ..." describing each step; exit status 0 when every check passed.
 */
#include "pfgpu.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Clauses {
    uint32_t max_var = 0;
    std::vector<uint32_t> lits;
    std::vector<uint64_t> off{0};
    uint64_t size() const { return off.size() - 1; }
};

struct Result {
    pfg_result_sizes sz{};
    std::vector<uint32_t> lits, units, pending, stack;
    std::vector<uint64_t> off, rends;
    std::vector<uint8_t> learnt, usage, elim;
    std::vector<uint32_t> lbd;
    void size_from(const pfg_result_sizes& s) {
        sz = s;
        lits.resize(s.literals);
        off.resize(s.clauses + 1);
        learnt.resize(s.clauses);
        lbd.resize(s.clauses);
        usage.resize(s.clauses);
        elim.resize(s.max_var + 1);
        units.resize(s.units);
        pending.resize(s.pending_units);
        stack.resize(s.stack_words);
        rends.resize(s.rounds);
    }
    /* clauses as sorted literal lists, in sorted order */
    std::vector<std::vector<uint32_t>> canonical() const {
        std::vector<std::vector<uint32_t>> cs;
        for (uint64_t i = 0; i + 1 < off.size(); i++) {
            std::vector<uint32_t> c(lits.begin() + off[i], lits.begin() + off[i + 1]);
            std::sort(c.begin(), c.end());
            c.push_back(learnt[i]);
            cs.push_back(c);
        }
        std::sort(cs.begin(), cs.end());
        return cs;
    }
};

bool g_ok = true;

void check(bool cond, const char* what) {
    printf("result %s %s\n", what, cond ? "ok" : "FAILED");
    if (!cond) g_ok = false;
}

int die(const char* what, int rc, const char* msg) {
    printf("result %s FAILED rc=%d %s\n", what, rc, msg ? msg : "");
    return 1;
}

/* Root assignment of the unit clauses: returns false on a conflict. */
bool root_propagate(const Clauses& in, const std::vector<uint32_t>& units, Clauses& out, std::vector<int8_t>& val) {
    val.assign(in.max_var + 1, -1);
    std::vector<uint32_t> queue(units);
    std::vector<char> alive(in.size(), 1);
    while (!queue.empty()) {
        for (uint32_t u : queue) {
            const int8_t want = (u & 1) ? 0 : 1;
            if (val[u >> 1] == -1) val[u >> 1] = want;
            else if (val[u >> 1] != want) return false;
        }
        queue.clear();
        for (uint64_t i = 0; i < in.size(); i++) {
            if (!alive[i]) continue;
            uint32_t free_lit = 0, nfree = 0;
            bool sat = false;
            for (uint64_t k = in.off[i]; k < in.off[i + 1]; k++) {
                const uint32_t l = in.lits[k];
                const int8_t v = val[l >> 1];
                if (v == -1) { free_lit = l; nfree++; }
                else if (v == ((l & 1) ? 0 : 1)) { sat = true; break; }
            }
            if (sat) { alive[i] = 0; continue; }
            if (nfree == 0) return false;
            if (nfree == 1) { queue.push_back(free_lit); alive[i] = 0; }
        }
    }
    out = Clauses();
    out.max_var = in.max_var;
    for (uint64_t i = 0; i < in.size(); i++) {
        if (!alive[i]) continue;
        for (uint64_t k = in.off[i]; k < in.off[i + 1]; k++)
            if (val[in.lits[k] >> 1] == -1) out.lits.push_back(in.lits[k]);
        out.off.push_back(out.lits.size());
    }
    return true;
}

template <class T>
void put_vec(FILE* f, const std::vector<T>& v) {
    if (!v.empty()) fwrite(v.data(), sizeof(T), v.size(), f);
}
template <class T>
void put(FILE* f, T v) { fwrite(&v, sizeof(T), 1, f); }

void put_head(FILE* f, uint32_t max_var, uint32_t status) {
    fwrite("PFREFDMP", 1, 8, f);
    put<uint32_t>(f, 1);
    put<uint32_t>(f, max_var);
    put<uint32_t>(f, status);
}

void write_input(const std::string& path, const Clauses& c) {
    FILE* f = fopen(path.c_str(), "wb");
    put_head(f, c.max_var, 0);
    const uint64_t n = c.size();
    put<uint64_t>(f, n);
    put<uint64_t>(f, c.lits.size());
    put_vec(f, c.off);
    put_vec(f, c.lits);
    put_vec(f, std::vector<uint8_t>(n, 0));
    put_vec(f, std::vector<uint32_t>(n, 0));
    put_vec(f, std::vector<uint8_t>(n, 0));
    fclose(f);
}

void write_output(const std::string& path, const Result& r, int status) {
    FILE* f = fopen(path.c_str(), "wb");
    put_head(f, r.sz.max_var, (uint32_t)status);
    put<uint64_t>(f, r.sz.clauses);
    put<uint64_t>(f, r.sz.literals);
    put_vec(f, r.off);
    put_vec(f, r.lits);
    put_vec(f, r.learnt);
    put_vec(f, r.lbd);
    put_vec(f, r.usage);
    put_vec(f, r.elim);
    put<uint64_t>(f, r.units.size());
    put_vec(f, r.units);
    put<uint64_t>(f, r.pending.size());
    put_vec(f, r.pending);
    put<uint64_t>(f, r.stack.size());
    put_vec(f, r.stack);
    put<uint32_t>(f, (uint32_t)r.rends.size());
    fclose(f);
}

void write_dimacs(const std::string& path, uint32_t max_var, const std::vector<uint32_t>& lits,
                  const std::vector<uint64_t>& off, const std::vector<uint32_t>& units) {
    FILE* f = fopen(path.c_str(), "w");
    fprintf(f, "p cnf %u %llu\n", max_var, (unsigned long long)(off.size() - 1 + units.size()));
    for (uint64_t i = 0; i + 1 < off.size(); i++) {
        for (uint64_t k = off[i]; k < off[i + 1]; k++)
            fprintf(f, "%s%u ", (lits[k] & 1) ? "-" : "", lits[k] >> 1);
        fprintf(f, "0\n");
    }
    for (uint32_t u : units) fprintf(f, "%s%u 0\n", (u & 1) ? "-" : "", u >> 1);
    fclose(f);
}

/* runs `cmd file`, returns 10/20/0 and the model (value[v] in {0,1}) */
int run_solver(const std::string& prog, const std::string& file, const std::string& opts, uint32_t nvars,
               std::vector<uint8_t>& model) {
    model.assign(nvars + 1, 0);
    const std::string line = prog + " " + file + opts + " 2>/dev/null";
    FILE* p = popen(line.c_str(), "r");
    if (!p) return 0;
    int status = 0;
    std::string buf;
    char chunk[4096];
    while (fgets(chunk, sizeof chunk, p)) buf += chunk;
    pclose(p);
    size_t pos = 0;
    while (pos < buf.size()) {
        size_t e = buf.find('\n', pos);
        if (e == std::string::npos) e = buf.size();
        std::string l = buf.substr(pos, e - pos);
        pos = e + 1;
        /* drop terminal colour escapes */
        std::string clean;
        for (size_t i = 0; i < l.size(); i++) {
            if (l[i] == '\x1b') { while (i < l.size() && l[i] != 'm') i++; continue; }
            clean += l[i];
        }
        if (clean.rfind("s SATISFIABLE", 0) == 0) status = 10;
        else if (clean.rfind("s UNSATISFIABLE", 0) == 0) status = 20;
        else if (!clean.empty() && clean[0] == 'v') {
            const char* s = clean.c_str() + 1;
            char* end = nullptr;
            for (;;) {
                long x = strtol(s, &end, 10);
                if (end == s) break;
                s = end;
                if (x > 0 && (uint64_t)x <= nvars) model[x] = 1;
            }
        }
    }
    return status;
}

bool download(pfg_ctx* ctx, Result& r) {
    pfg_result_sizes sz;
    if (pfg_result_sizes_get(ctx, &sz)) return false;
    r.size_from(sz);
    return pfg_download(ctx, r.lits.data(), r.off.data(), r.learnt.data(), r.lbd.data(), r.usage.data(),
                        r.elim.data(), r.units.data(), r.pending.data(), r.stack.data(), r.rends.data()) == PFG_OK;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s in.cnf work-dir [solver [options...]]\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[2];
    /* solver program, then its options: run as `program file options...` */
    std::string solver, solver_opts;
    if (argc > 3) solver = argv[3];
    for (int i = 4; i < argc; i++) solver_opts += std::string(" ") + argv[i];

    /* ---- ingest ---- */
    pfg_dimacs* d = nullptr;
    if (pfg_dimacs_read(argv[1], &d) != PFG_OK) return die("dimacs", 0, d ? pfg_dimacs_error(d) : "");
    pfg_dimacs_info info;
    pfg_dimacs_get_info(d, &info);
    Clauses orig;
    orig.max_var = info.max_var;
    orig.lits.resize(info.num_literals);
    orig.off.resize(info.num_clauses + 1);
    std::vector<uint32_t> in_units(info.num_units);
    pfg_dimacs_copy(d, orig.lits.data(), orig.off.data(), in_units.data());
    pfg_dimacs_free(d);
    printf("result dimacs ok vars=%u clauses=%llu units=%llu\n", info.max_var, (unsigned long long)info.num_clauses,
           (unsigned long long)info.num_units);
    Clauses cnf;
    std::vector<int8_t> root;
    if (info.status == PFG_UNSAT || !root_propagate(orig, in_units, cnf, root)) {
        printf("result status 20 (root conflict)\n");
        return 0;
    }
    write_input(dir + "/simp.in", cnf);

    /* ---- simplify: the host adapter's call sequence ---- */
    pfg_options opts;
    pfg_default_options(&opts);
    pfg_resolve_options(&opts);
    pfg_ctx* ctx = nullptr;
    int rc = pfg_create(&ctx, &opts, 0);
    if (rc) return die("pfg_create", rc, "");
    rc = pfg_upload(ctx, cnf.max_var, cnf.size(), cnf.lits.data(), cnf.off.data(), nullptr, nullptr, nullptr,
                    nullptr, nullptr, nullptr);
    if (rc) return die("pfg_upload", rc, pfg_last_error(ctx));
    pfg_stats st;
    rc = pfg_simplify(ctx, &st);
    if (rc) return die("pfg_simplify", rc, pfg_last_error(ctx));
    Result single;
    if (!download(ctx, single)) return die("pfg_download", 0, pfg_last_error(ctx));
    pfg_destroy(ctx);
    write_output(dir + "/simp.out", single, st.status);
    printf("result simplify ok status=%d rounds=%d clauses=%llu->%llu eliminated=%llu\n", st.status, st.rounds,
           (unsigned long long)st.clauses_in, (unsigned long long)st.clauses_out,
           (unsigned long long)st.eliminated);

    /* ---- the same CNF twice in one batch ---- */
    {
        pfg_ctx* b = nullptr;
        rc = pfg_create(&b, &opts, 0);
        if (rc) return die("pfg_create batch", rc, "");
        pfg_instance ins[2];
        memset(ins, 0, sizeof ins);
        for (auto& x : ins) {
            x.max_var = cnf.max_var;
            x.num_clauses = cnf.size();
            x.lits = cnf.lits.data();
            x.cls_off = cnf.off.data();
        }
        rc = pfg_batch_upload(b, 2, ins);
        if (rc) return die("pfg_batch_upload", rc, pfg_last_error(b));
        pfg_stats bt;
        rc = pfg_simplify(b, &bt);
        if (rc) return die("pfg_simplify batch", rc, pfg_last_error(b));
        check(pfg_batch_size(b) == 2, "batch_size");
        for (uint32_t i = 0; i < 2; i++) {
            pfg_result_sizes sz;
            pfg_batch_result_sizes(b, i, &sz);
            Result r;
            r.size_from(sz);
            rc = pfg_batch_download(b, i, r.lits.data(), r.off.data(), r.learnt.data(), r.lbd.data(), r.usage.data(),
                                    r.elim.data(), r.units.data(), r.pending.data(), r.stack.data(), r.rends.data());
            check(rc == PFG_OK && r.canonical() == single.canonical() && r.elim == single.elim &&
                      r.stack.size() == single.stack.size(),
                  i ? "batch_instance_1" : "batch_instance_0");
        }
        pfg_destroy(b);
    }

    /* ---- two contexts simplified at once (pfg_simplify_many) ---- */
    {
        pfg_ctx* m[2] = {nullptr, nullptr};
        for (auto& x : m) {
            rc = pfg_create(&x, &opts, 0);
            if (rc) return die("pfg_create many", rc, "");
            rc = pfg_upload(x, cnf.max_var, cnf.size(), cnf.lits.data(), cnf.off.data(), nullptr, nullptr, nullptr,
                            nullptr, nullptr, nullptr);
            if (rc) return die("pfg_upload many", rc, pfg_last_error(x));
        }
        pfg_stats ms[2];
        float dev_ms = 0;
        rc = pfg_simplify_many(m, 2, ms, &dev_ms);
        if (rc) return die("pfg_simplify_many", rc, pfg_last_error(m[0]));
        check(dev_ms > 0.0f, "many_device_ms");
        for (int j = 0; j < 2; j++) {
            Result r;
            if (!download(m[j], r)) return die("pfg_download many", 0, pfg_last_error(m[j]));
            check(r.canonical() == single.canonical() && r.elim == single.elim && ms[j].rounds == st.rounds,
                  j ? "many_context_1" : "many_context_0");
            pfg_destroy(m[j]);
        }
    }

    /* ---- one job through the serving loop ---- */
    {
        pfg_server* srv = nullptr;
        rc = pfg_server_create(&srv, &opts, size_t(4) << 30, 2, 8);
        if (rc) return die("pfg_server_create", rc, srv ? pfg_server_last_error(srv) : "");
        pfg_instance job;
        memset(&job, 0, sizeof job);
        job.max_var = cnf.max_var;
        job.num_clauses = cnf.size();
        job.lits = cnf.lits.data();
        job.cls_off = cnf.off.data();
        uint64_t ticket = 0;
        rc = pfg_server_submit(srv, &job, &ticket);
        if (rc) return die("pfg_server_submit", rc, pfg_server_last_error(srv));
        pfg_job_info ji;
        do { rc = pfg_server_poll(srv, ticket, 1000, &ji); } while (rc == PFG_PENDING);
        if (rc) return die("pfg_server_poll", rc, pfg_server_last_error(srv));
        Result r;
        r.size_from(ji.sizes);
        rc = pfg_server_fetch(srv, ticket, r.lits.data(), r.off.data(), r.learnt.data(), r.lbd.data(), r.usage.data(),
                              r.elim.data(), r.units.data(), r.pending.data(), r.stack.data(), r.rends.data());
        check(rc == PFG_OK && ji.rc == PFG_OK && r.canonical() == single.canonical() && r.elim == single.elim,
              "server_job");
        pfg_server_destroy(srv);
    }

    if (st.status == PFG_UNSAT) {
        printf("result status 20\n");
        return g_ok ? 0 : 1;
    }

    /* ---- write-back: map the active variables, solve, extend ---- */
    std::vector<uint32_t> new_of_old(cnf.max_var + 1), old_of_new(cnf.max_var + 1);
    uint32_t nv = 0;
    rc = pfg_map_vars(cnf.max_var, single.elim.data(), new_of_old.data(), old_of_new.data(), &nv);
    if (rc) return die("pfg_map_vars", rc, "");
    std::vector<uint32_t> mlits(single.lits.size()), munits(single.pending.size());
    if (!mlits.empty() && pfg_map_lits(new_of_old.data(), cnf.max_var, mlits.size(), single.lits.data(), mlits.data()))
        return die("pfg_map_lits", 0, "");
    if (!munits.empty() &&
        pfg_map_lits(new_of_old.data(), cnf.max_var, munits.size(), single.pending.data(), munits.data()))
        return die("pfg_map_lits units", 0, "");
    const std::string mapped = dir + "/mapped.cnf";
    write_dimacs(mapped, nv, mlits, single.off, munits);
    printf("result mapped ok vars=%u clauses=%llu\n", nv, (unsigned long long)single.sz.clauses);
    if (solver.empty()) return g_ok ? 0 : 1;

    std::vector<uint8_t> mmodel;
    int status = 10;
    if (single.sz.clauses || !munits.empty()) status = run_solver(solver, mapped, solver_opts, nv, mmodel);
    else mmodel.assign(nv + 1, 0);
    printf("result solver status %d\n", status);
    if (status != 10) {
        printf("result status %d\n", status);
        return g_ok && status == 20 ? 0 : 1;
    }
    std::vector<uint8_t> value(cnf.max_var + 1, 0);
    for (uint32_t v = 1; v <= nv; v++) value[old_of_new[v]] = mmodel[v];
    for (uint32_t v = 1; v <= cnf.max_var; v++)
        if (root[v] >= 0) value[v] = (uint8_t)root[v];
    for (uint32_t u : single.units) value[u >> 1] = (u & 1) ? 0 : 1;
    rc = pfg_extend_model(single.stack.size(), single.stack.data(), cnf.max_var, value.data());
    if (rc) return die("pfg_extend_model", rc, "");
    /* every original clause, units included, must hold */
    bool sat = true;
    for (uint64_t i = 0; i < orig.size() && sat; i++) {
        bool any = false;
        for (uint64_t k = orig.off[i]; k < orig.off[i + 1] && !any; k++)
            any = value[orig.lits[k] >> 1] == ((orig.lits[k] & 1) ? 0 : 1);
        sat = any;
    }
    for (uint32_t u : in_units) sat = sat && value[u >> 1] == ((u & 1) ? 0 : 1);
    check(sat, "model_verified");
    printf("result status 10\n");
    return g_ok ? 0 : 1;
}
