/*
 * time_main.cpp - times the reference's own CPU simplifier on one DIMACS file
 * (TEST AND BASELINE INFRASTRUCTURE ONLY).
 *
 * Built by oracle/ref_build.py against the unmodified reference CPU sources
 * (src/cpu) in place of their main (src/cpu/main.cpp:28-98). The options are
 * parsed the same way (parseArguments); the solver is constructed from the
 * file (parsing, untimed); then Solver::sigmify (src/cpu/simplify.cpp:115)
 * runs once under a steady clock, as Solver::solve would run it before the
 * search (solver.cpp:147-149: initLimits, then sigmify).
 *
 * Work count: the link step wraps Solver::SUB (src/cpu/elimination.cpp) with
 * `-Wl,--wrap`, so each call first adds the live clauses entering that
 * SUB+BVE round (inf.nClauses, simplify.cpp:176-183) to a counter. That is
 * the same work unit the GPU engine reports (clauses entering SUB+BVE per
 * round). Nothing in the reference is changed.
 *
 * Output: one line "pfref_cpu clauses_in=C processed=P rounds=R seconds=T
 * status=S" on stdout. A conflict found while simplifying ends the process
 * inside the reference (killSolver, control.cpp); an exit handler then
 * prints the line with status=20 and the time until then.
 */
#include "control.h"
#include "solver.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

using namespace ParaFROST;

bool quiet_en = false;
bool competition_en = false;
int verbose = -1;

namespace {
uint64_t g_processed = 0, g_rounds = 0, g_clauses_in = 0;
bool g_timing = false, g_printed = false;
std::chrono::steady_clock::time_point g_t0;

void print_line(int status) {
    if (g_printed) return;
    g_printed = true;
    double s = g_timing ? std::chrono::duration<double>(std::chrono::steady_clock::now() - g_t0).count() : 0.0;
    printf("pfref_cpu clauses_in=%llu processed=%llu rounds=%llu seconds=%.9f status=%d\n",
           (unsigned long long)g_clauses_in, (unsigned long long)g_processed, (unsigned long long)g_rounds, s,
           status);
    fflush(stdout);
}

void on_exit_handler() { print_line(20); }
}  // namespace

extern "C" void __real__ZN9ParaFROST6Solver3SUBEv(Solver* self);
extern "C" void __wrap__ZN9ParaFROST6Solver3SUBEv(Solver* self) {
    g_processed += inf.nClauses;
    g_rounds++;
    __real__ZN9ParaFROST6Solver3SUBEv(self);
}

class Timer : public Solver {
public:
    explicit Timer(const std::string& path) : Solver(path) {}
    uint64_t clauses() const { return uint64_t(stats.clauses.original) + uint64_t(stats.clauses.learnt); }
    int run() {
        initLimits();
        if (!UNSOLVED(cnfstate) || !stats.clauses.original) return cnfstate == SAT ? 10 : 20;
        g_t0 = std::chrono::steady_clock::now();
        g_timing = true;
        sigmify();
        return UNSOLVED(cnfstate) ? 0 : (cnfstate == SAT ? 10 : 20);
    }
};

int main(int argc, char** argv) {
    /* usage: pfref_cpu_time <formula.cnf> [reference options...] */
    if (argc < 2) {
        fprintf(stderr, "usage: %s formula.cnf [options]\n", argv[0]);
        return 2;
    }
    BOOL_OPT opt_quiet_en("quiet", "enable quiet mode, same as verbose=0", false);
    INT_OPT opt_verbose("verbose", "set the verbosity", 0, INT32R(0, 4));
    parseArguments(argc, argv);
    quiet_en = opt_quiet_en, verbose = opt_verbose;
    if (!verbose) quiet_en = true;
    atexit(on_exit_handler);
    Timer* t = new Timer(argv[1]);
    solver = t;
    g_clauses_in = t->clauses();
    const int status = t->run();
    print_line(status);
    return 0;
}
