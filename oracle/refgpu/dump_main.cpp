/*
 * dump_main.cpp - drives the reference GPU simplifier on one DIMACS file and
 * writes its input and results in binary form (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/ref_gpu_build.py against the unmodified reference sources
 * (src/gpu) and the cuArena stand-in in oracle/refgpu/cuarena. It replaces
 * the reference's main (src/gpu/main.cpp:38-98): the options are parsed the
 * same way (parseArguments), the solver is constructed from the file (parse
 * + root propagation, src/gpu/solver.cpp:42-48), then instead of solve() it
 *
 *  1. takes the clause database to the state Solver::simplifying hands to
 *     awaken (rootify + shrinkTop, src/gpu/simplify.cu:143-145) and writes it
 *     (originals, then learnts, in the order awaken extracts them,
 *     simplify.cu:106-107) to <out>.in;
 *  2. runs Solver::simplify(true) (simplify.cu:57), which leaves the
 *     simplified clauses in the host mirror hcnf (cacheCNF, cnf.cu:200-236);
 *  3. fetches the model-reconstruction stack (cacheResolved, transfer.cu:83),
 *     the eliminated bytes (cacheEliminated, transfer.cu:69) and the units
 *     of the last round that were not propagated, and writes them with the
 *     clauses and the literals the device propagation assigned to <out>.out.
 *
 * When device propagation finds a conflict the reference ends the process
 * (prop -> killSolver -> exit, src/gpu/simplify.cu:168, control.cpp:270); an
 * exit handler then writes <out>.out with the UNSAT status only.
 *
 * File layout (little endian): "PFREFDMP", u32 version = 1, u32 max_var,
 * u32 status (0 unknown, 10 SAT, 20 UNSAT), then for a CNF section:
 * u64 n, u64 nlits, u64 off[n+1], u32 lits[nlits], u8 learnt[n], u32 lbd[n],
 * u8 usage[n]; then (.out only) u8 eliminated[max_var+1], u64 nassigned,
 * u32 assigned[nassigned] (root trail literals after simplify that were not
 * on the trail before it), u64 npending, u32 pending[npending],
 * u64 nstack, u32 stack[nstack], u32 phases_run.
 */
#include "control.hpp"
#include "solver.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace ParaFROST;

bool quiet_en = false;
int verbose = -1;

namespace {

struct CnfArrays {
    std::vector<uint64_t> off{0};
    std::vector<uint32_t> lits;
    std::vector<uint8_t> learnt, usage;
    std::vector<uint32_t> lbd;
    void add(const uint32_t* l, int n, bool is_learnt, uint32_t b, uint32_t u) {
        lits.insert(lits.end(), l, l + n);
        off.push_back(lits.size());
        learnt.push_back(is_learnt ? 1 : 0);
        lbd.push_back(b);
        usage.push_back(uint8_t(u));
    }
};

template <class T>
void put(FILE* f, const T& v) { fwrite(&v, sizeof(T), 1, f); }
template <class T>
void put_vec(FILE* f, const std::vector<T>& v) {
    if (!v.empty()) fwrite(v.data(), sizeof(T), v.size(), f);
}

void put_cnf(FILE* f, const CnfArrays& c) {
    put<uint64_t>(f, c.learnt.size());
    put<uint64_t>(f, c.lits.size());
    put_vec(f, c.off);
    put_vec(f, c.lits);
    put_vec(f, c.learnt);
    put_vec(f, c.lbd);
    put_vec(f, c.usage);
}

void put_head(FILE* f, uint32_t max_var, uint32_t status) {
    fwrite("PFREFDMP", 1, 8, f);
    put<uint32_t>(f, 1);
    put<uint32_t>(f, max_var);
    put<uint32_t>(f, status);
}

std::string g_out;
bool g_done = false;
uint32_t g_max_var = 0;

void write_unsat_on_exit() {
    if (g_done || g_out.empty()) return;
    FILE* f = fopen((g_out + ".out").c_str(), "wb");
    if (!f) return;
    put_head(f, g_max_var, 20);
    fclose(f);
}

}  // namespace

class Dumper : public Solver {
public:
    explicit Dumper(const std::string& path) : Solver(path) {}

    uint32_t max_var() const { return inf.maxVar; }

    /* The database in the state Solver::simplifying hands to awaken. */
    void prepare_and_dump_input(const std::string& out) {
        initLimits();
        rootify();
        shrinkTop(false);
        CnfArrays in;
        auto take = [&](BCNF& list) {
            forall_cnf(list, i) {
                const C_REF r = *i;
                if (cm.deleted(r)) continue;
                CLAUSE& c = cm[r];
                in.add(c.data(), c.size(), c.learnt(), c.learnt() ? c.lbd() : 0, c.learnt() ? c.usage() : 0);
            }
        };
        take(orgs);
        take(learnts);
        trail_before.assign(trail.data(), trail.data() + trail.size());
        FILE* f = fopen((out + ".in").c_str(), "wb");
        if (!f) { fprintf(stderr, "cannot write %s.in\n", out.c_str()); exit(2); }
        put_head(f, inf.maxVar, 0);
        put_cnf(f, in);
        fclose(f);
    }

    void run_and_dump_output(const std::string& out) {
        simplify(true);
        SYNCALL;
        uint32_t status = cnfstate == UNSAT ? 20 : (cnfstate == SAT ? 10 : 0);
        /* clauses left in the host mirror (skip_transfer_to_host path) */
        CnfArrays res;
        if (status == 0 && hcnf) {
            for (uint32 i = 0; i < hcnf->size(); i++) {
                SCLAUSE& s = hcnf->clause(i);
                if (s.deleted()) continue;
                res.add(s.data(), s.size(), s.learnt(), s.lbd(), s.usage());
            }
        }
        /* eliminated bytes: cached by simplifying except on the SAT return */
        cacheEliminated(streams[5]);
        SYNCALL;
        std::vector<uint8_t> elim(vars->cachedEliminated, vars->cachedEliminated + inf.maxVar + 1);
        /* model-reconstruction stack: cacheResolved runs only in newBeginning
           and on the SAT return, so fetch it here when simplifying did not */
        if (status == 0) { cacheResolved(streams[2]); SYNCALL; }
        std::vector<uint32_t> stack(model.resolved.data(), model.resolved.data() + model.resolved.size());
        /* units the last round produced that no later propagation consumed */
        std::vector<uint32_t> pending;
        {
            cuVecU tmp;
            CHECK(cudaMemcpy(&tmp, vars->units, sizeof(cuVecU), cudaMemcpyDeviceToHost));
            if (tmp.size()) {
                pending.resize(tmp.size());
                CHECK(cudaMemcpy(pending.data(), tmp.data(), tmp.size() * sizeof(uint32), cudaMemcpyDeviceToHost));
            }
        }
        std::vector<uint32_t> assigned;
        {
            std::vector<uint8_t> before(2 * (size_t(inf.maxVar) + 1), 0);
            for (uint32_t l : trail_before) before[l] = 1;
            for (uint32 k = 0; k < trail.size(); k++)
                if (!before[trail[k]]) assigned.push_back(trail[k]);
        }
        FILE* f = fopen((out + ".out").c_str(), "wb");
        if (!f) { fprintf(stderr, "cannot write %s.out\n", out.c_str()); exit(2); }
        put_head(f, inf.maxVar, status);
        put_cnf(f, res);
        put_vec(f, elim);
        put<uint64_t>(f, assigned.size());
        put_vec(f, assigned);
        put<uint64_t>(f, pending.size());
        put_vec(f, pending);
        put<uint64_t>(f, stack.size());
        put_vec(f, stack);
        put<uint32_t>(f, uint32_t(phase));
        fclose(f);
        g_done = true;
    }

private:
    std::vector<uint32_t> trail_before;
};

int main(int argc, char** argv) {
    /* usage: pfref_gpu <formula.cnf> <out-prefix> [reference options...] */
    if (argc < 3) {
        fprintf(stderr, "usage: %s formula.cnf out-prefix [options]\n", argv[0]);
        return 2;
    }
    g_out = argv[2];
    std::vector<char*> args;
    args.push_back(argv[0]);
    args.push_back(argv[1]);
    for (int i = 3; i < argc; i++) args.push_back(argv[i]);
    BOOL_OPT opt_quiet_en("quiet", "enable quiet mode, same as verbose=0", false);
    INT_OPT opt_verbose("verbose", "set the verbosity", 0, INT32R(0, 4));
    int nargs = int(args.size());
    parseArguments(nargs, args.data());
    quiet_en = opt_quiet_en, verbose = opt_verbose;
    if (!verbose) quiet_en = true;
    atexit(write_unsat_on_exit);
    Dumper* d = new Dumper(argv[1]);
    init_solver(d);
    g_max_var = d->max_var();
    d->prepare_and_dump_input(g_out);
    d->run_and_dump_output(g_out);
    return 0;
}
