// Serving loop: simplification jobs that arrive over time, admitted by an
// arena memory budget and run as batches on several concurrent slots.
//
// No counterpart in the reference (which simplifies the one CNF of its
// Solver). A job is an instance copied at submit time. Workers -- one thread,
// one engine context and one stream each -- take the waiting jobs in arrival
// order while their estimated device footprint fits what the budget has left
// and simplify them as one batch (pfg_batch_upload / pfg_simplify /
// pfg_batch_download). A worker that finishes returns its jobs' memory to the
// budget and wakes the others, so jobs that arrive while other batches run
// start as soon as a slot and memory are free, and the batches of different
// slots overlap on the device.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "pfgpu.h"

namespace {

uint64_t now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Results of one batch, every instance back to back (pfg_batch_download_all);
// each job of the batch keeps a reference and its offsets.
struct BatchResult {
    std::vector<uint32_t> lits, lbd, units, pending, stack;
    std::vector<uint64_t> off, rends;
    std::vector<uint8_t> learnt, usage, elim;
};

struct Slice {
    uint64_t lits = 0, cls = 0, off = 0, elim = 0, units = 0, pending = 0, stack = 0, rends = 0;
};

struct Job {
    uint64_t ticket = 0;
    // the instance (owned copy, released once uploaded)
    uint32_t max_var = 0;
    uint64_t num_clauses = 0;
    std::vector<uint32_t> lits, lbd, vorg;
    std::vector<uint64_t> off;
    std::vector<uint8_t> learnt, usage, var_state, assumed;
    uint64_t est = 0;
    bool done = false;
    pfg_job_info info{};
    std::shared_ptr<BatchResult> res;   // results, from `at`
    std::vector<uint8_t> proof;         // binary DRAT lines of the job (proof_en)
    Slice at;
};

template <typename T>
void copy_in(std::vector<T>& dst, const T* src, uint64_t n) {
    if (src) dst.assign(src, src + n); else dst.clear();
}

template <typename T>
const T* ptr_or_null(const std::vector<T>& v) { return v.empty() ? nullptr : v.data(); }

// Device bytes an instance needs inside one batch: the clause store at the
// capacities of awaken (originals may double the clauses and literals), the
// occurrence table, ~30 per-variable arrays, the unit / trail / stack regions
// and sort and scan scratch, with a quarter on top for pool rounding.
uint64_t estimate(uint32_t V, uint64_t C, uint64_t L) {
    const uint64_t b = 2 * C * 16          // clause headers
                     + 4 * (2 * L + 3 * C) // literals with added-clause headroom
                     + 12 * L              // occurrence lists with growth
                     + 2 * (2ull * V + 2) * 4 * 5   // list sizes, offsets, cursors, histogram
                     + 136ull * (V + 1)    // per-variable arrays
                     + 16 * (C + L)        // model stack region
                     + 12ull * (V + 1)     // units and trail regions
                     + 48 * C;             // sort keys and scratch
    return b + b / 4 + (1ull << 20);
}

// the checks of the engine's upload, so one bad job cannot fail a whole batch
bool valid_job(const pfg_instance& q, std::string& why) {
    if (q.max_var == 0 || q.max_var > 0x7FFFFFF0u || (q.num_clauses && (!q.lits || !q.cls_off))) {
        why = "invalid arguments";
        return false;
    }
    if (!q.num_clauses) return true;
    if (q.cls_off[0] != 0) { why = "cls_off[0] must be 0"; return false; }
    const uint64_t nlits = q.cls_off[q.num_clauses];
    std::vector<uint64_t> seen((size_t)q.max_var + 1, ~0ull);
    for (uint64_t i = 0; i < q.num_clauses; i++) {
        const uint64_t b = q.cls_off[i], e = q.cls_off[i + 1];
        if (e < b + 2 || e > nlits) { why = "clause " + std::to_string(i) + " has fewer than 2 literals"; return false; }
        for (uint64_t k = b; k < e; k++) {
            const uint32_t v = q.lits[k] >> 1;
            if (v == 0 || v > q.max_var) { why = "literal out of range in clause " + std::to_string(i); return false; }
            if (seen[v] == i) { why = "repeated variable in clause " + std::to_string(i); return false; }
            seen[v] = i;
        }
    }
    return true;
}

}  // namespace

struct pfg_server {
    pfg_options opts{};
    size_t budget = 0;
    uint32_t slots = 1, max_batch = 1;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
    uint64_t next_ticket = 1;
    uint64_t in_use = 0;
    uint64_t batches_in_flight = 0, jobs_in_flight = 0;
    bool stopping = false;
    pfg_server_stats st{};
    std::vector<pfg_ctx*> ctx;
    std::vector<std::thread> workers;
    std::string err;
};

namespace {

void run_batch(pfg_server* s, pfg_ctx* ctx, uint32_t slot, std::vector<Job*>& batch) {
    const uint32_t n = (uint32_t)batch.size();
    std::vector<pfg_instance> ins(n);
    for (uint32_t i = 0; i < n; i++) {
        Job* j = batch[i];
        pfg_instance& q = ins[i];
        std::memset(&q, 0, sizeof(q));
        q.max_var = j->max_var;
        q.num_clauses = j->num_clauses;
        q.lits = ptr_or_null(j->lits);
        q.cls_off = ptr_or_null(j->off);
        q.cls_learnt = ptr_or_null(j->learnt);
        q.cls_lbd = ptr_or_null(j->lbd);
        q.cls_usage = ptr_or_null(j->usage);
        q.var_state = ptr_or_null(j->var_state);
        q.assumed = ptr_or_null(j->assumed);
        q.vorg = ptr_or_null(j->vorg);
    }
    int rc = pfg_batch_upload(ctx, n, ins.data());
    for (Job* j : batch) {   // the device holds the instance now
        std::vector<uint32_t>().swap(j->lits);
        std::vector<uint64_t>().swap(j->off);
        std::vector<uint8_t>().swap(j->learnt);
        std::vector<uint32_t>().swap(j->lbd);
        std::vector<uint8_t>().swap(j->usage);
    }
    pfg_stats total;
    if (rc == PFG_OK) rc = pfg_simplify(ctx, &total);
    std::vector<pfg_result_sizes> z(n);
    auto res = std::make_shared<BatchResult>();
    if (rc == PFG_OK) rc = pfg_batch_result_sizes_all(ctx, z.data());
    if (rc == PFG_OK) {
        Slice tot;
        for (uint32_t i = 0; i < n; i++) {
            batch[i]->at = tot;
            tot.lits += z[i].literals;
            tot.cls += z[i].clauses;
            tot.off += z[i].clauses + 1;
            tot.elim += (uint64_t)z[i].max_var + 1;
            tot.units += z[i].units;
            tot.pending += z[i].pending_units;
            tot.stack += z[i].stack_words;
            tot.rends += z[i].rounds;
        }
        res->lits.resize(tot.lits); res->off.resize(tot.off); res->learnt.resize(tot.cls);
        res->lbd.resize(tot.cls); res->usage.resize(tot.cls); res->elim.resize(tot.elim);
        res->units.resize(tot.units); res->pending.resize(tot.pending); res->stack.resize(tot.stack);
        res->rends.resize(tot.rends);
        rc = pfg_batch_download_all(ctx, res->lits.data(), res->off.data(), res->learnt.data(), res->lbd.data(),
                                    res->usage.data(), res->elim.data(), res->units.data(), res->pending.data(),
                                    res->stack.data(), res->rends.data());
    }
    for (uint32_t i = 0; i < n; i++) {
        Job* j = batch[i];
        pfg_job_info& in = j->info;
        in.rc = rc;
        in.batch_size = n;
        in.slot = slot;
        if (rc != PFG_OK) continue;
        in.sizes = z[i];
        j->res = res;
        pfg_stats st;
        int r = pfg_batch_stats(ctx, i, &st);
        if (r == PFG_OK && z[i].proof_bytes) {    // the instance's own proof, as pfg_batch_download_proof gives it
            j->proof.resize(z[i].proof_bytes);
            r = pfg_batch_download_proof(ctx, i, j->proof.data());
        }
        in.rc = r;
        if (r == PFG_OK) {
            in.status = st.status;
            in.clauses_processed = st.clauses_processed;
        }
    }
}

void worker(pfg_server* s, uint32_t slot) {
    cudaSetDevice(s->device);
    pfg_ctx* ctx = s->ctx[slot];
    for (;;) {
        std::vector<Job*> batch;
        uint64_t charged = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (s->queue.empty()) {
                    if (s->stopping) return;
                    s->cv_work.wait(lk);
                    continue;
                }
                // admission in arrival order while the budget allows; a job
                // larger than the whole budget runs alone on an idle device
                while (!s->queue.empty() && batch.size() < s->max_batch) {
                    Job* j = s->queue.front();
                    const bool fits = s->in_use + charged + j->est <= s->budget;
                    const bool alone = s->in_use == 0 && batch.empty();
                    if (!fits && !alone) break;
                    charged += j->est;
                    batch.push_back(j);
                    s->queue.pop_front();
                    if (!fits) break;
                }
                if (!batch.empty()) break;
                s->cv_work.wait(lk);   // memory is held by running batches
            }
            const uint64_t t = now_ns();
            for (Job* j : batch) j->info.t_admit_ns = t;
            s->in_use += charged;
            s->batches_in_flight++;
            s->jobs_in_flight += batch.size();
            s->st.admitted += batch.size();
            s->st.batches++;
            s->st.max_in_flight_batches = std::max<uint64_t>(s->st.max_in_flight_batches, s->batches_in_flight);
            s->st.max_jobs_in_flight = std::max<uint64_t>(s->st.max_jobs_in_flight, s->jobs_in_flight);
            s->st.peak_est_bytes = std::max<uint64_t>(s->st.peak_est_bytes, s->in_use);
        }
        run_batch(s, ctx, slot, batch);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const uint64_t t = now_ns();
            for (Job* j : batch) {
                j->info.t_done_ns = t;
                j->done = true;
            }
            s->in_use -= charged;
            s->batches_in_flight--;
            s->jobs_in_flight -= batch.size();
            s->st.done += batch.size();
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" int pfg_server_create(pfg_server** out, const pfg_options* opts, size_t arena_bytes, uint32_t slots,
                                 uint32_t max_batch) {
    if (!out || slots == 0 || slots > 64 || max_batch == 0) return PFG_INVALID;
    *out = nullptr;
    pfg_server* s = new pfg_server();
    if (opts) s->opts = *opts; else pfg_default_options(&s->opts);
    s->slots = slots;
    s->max_batch = max_batch;
    if (cudaGetDevice(&s->device) != cudaSuccess) { cudaGetLastError(); delete s; return PFG_CUDA_ERROR; }
    if (arena_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); delete s; return PFG_CUDA_ERROR; }
        arena_bytes = fr > (1ull << 30) ? fr - (1ull << 30) : fr / 2;
    }
    s->budget = arena_bytes;
    s->st.budget_bytes = arena_bytes;
    for (uint32_t i = 0; i < slots; i++) {
        pfg_ctx* c = nullptr;
        const int rc = pfg_create(&c, &s->opts, arena_bytes);
        if (rc != PFG_OK) {
            for (pfg_ctx* x : s->ctx) pfg_destroy(x);
            delete s;
            return rc;
        }
        s->ctx.push_back(c);
    }
    for (uint32_t i = 0; i < slots; i++) s->workers.emplace_back(worker, s, i);
    *out = s;
    return PFG_OK;
}

extern "C" int pfg_server_submit(pfg_server* s, const pfg_instance* q, uint64_t* ticket) {
    if (!s || !q || !ticket) return PFG_INVALID;
    std::string why;
    if (!valid_job(*q, why)) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->err = "invalid job: " + why;
        return PFG_INVALID;
    }
    std::unique_ptr<Job> j(new Job());
    const uint64_t C = q->num_clauses, L = C ? q->cls_off[C] : 0;
    j->max_var = q->max_var;
    j->num_clauses = C;
    copy_in(j->lits, q->lits, L);
    copy_in(j->off, q->cls_off, C ? C + 1 : 0);
    copy_in(j->learnt, q->cls_learnt, C);
    copy_in(j->lbd, q->cls_lbd, C);
    copy_in(j->usage, q->cls_usage, C);
    copy_in(j->var_state, q->var_state, (uint64_t)q->max_var + 1);
    copy_in(j->assumed, q->assumed, (uint64_t)q->max_var + 1);
    copy_in(j->vorg, q->vorg, (uint64_t)q->max_var + 1);
    j->est = estimate(q->max_var, C, L);
    j->info.est_bytes = j->est;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) { s->err = "server is stopping"; return PFG_INVALID; }
        j->ticket = s->next_ticket++;
        j->info.t_submit_ns = now_ns();
        *ticket = j->ticket;
        s->queue.push_back(j.get());
        s->jobs[j->ticket] = std::move(j);
        s->st.submitted++;
    }
    s->cv_work.notify_one();
    return PFG_OK;
}

extern "C" int pfg_server_poll(pfg_server* s, uint64_t ticket, int32_t wait_ms, pfg_job_info* info) {
    if (!s) return PFG_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return PFG_INVALID;
    Job* j = it->second.get();
    if (!j->done && wait_ms > 0)
        s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return j->done; });
    if (!j->done) return PFG_PENDING;
    if (info) *info = j->info;
    return PFG_OK;
}

extern "C" int pfg_server_fetch(pfg_server* s, uint64_t ticket, uint32_t* lits, uint64_t* cls_off,
                                uint8_t* cls_learnt, uint32_t* cls_lbd, uint8_t* cls_usage, uint8_t* eliminated,
                                uint32_t* units, uint32_t* pending_units, uint32_t* stack, uint64_t* round_ends) {
    if (!s) return PFG_INVALID;
    std::unique_ptr<Job> j;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(ticket);
        if (it == s->jobs.end()) return PFG_INVALID;
        if (!it->second->done) return PFG_PENDING;
        j = std::move(it->second);
        s->jobs.erase(it);
    }
    if (j->info.rc != PFG_OK) return j->info.rc;
    const pfg_result_sizes& z = j->info.sizes;
    const BatchResult& r = *j->res;
    const Slice& a = j->at;
    auto put = [](auto* dst, const auto& v, uint64_t from, uint64_t count) {
        if (dst && count) std::copy(v.begin() + from, v.begin() + from + count, dst);
    };
    put(lits, r.lits, a.lits, z.literals);
    put(cls_off, r.off, a.off, z.clauses + 1);
    put(cls_learnt, r.learnt, a.cls, z.clauses);
    put(cls_lbd, r.lbd, a.cls, z.clauses);
    put(cls_usage, r.usage, a.cls, z.clauses);
    put(eliminated, r.elim, a.elim, (uint64_t)z.max_var + 1);
    put(units, r.units, a.units, z.units);
    put(pending_units, r.pending, a.pending, z.pending_units);
    put(stack, r.stack, a.stack, z.stack_words);
    put(round_ends, r.rends, a.rends, z.rounds);
    return PFG_OK;
}

extern "C" int pfg_server_fetch_proof(pfg_server* s, uint64_t ticket, uint8_t* out) {
    if (!s) return PFG_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return PFG_INVALID;
    const Job& j = *it->second;
    if (!j.done) return PFG_PENDING;
    if (j.info.rc != PFG_OK) return j.info.rc;
    if (out && !j.proof.empty()) std::copy(j.proof.begin(), j.proof.end(), out);
    return PFG_OK;
}

extern "C" int pfg_server_stats_get(pfg_server* s, pfg_server_stats* st) {
    if (!s || !st) return PFG_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->st;
    return PFG_OK;
}

extern "C" const char* pfg_server_last_error(pfg_server* s) {
    if (!s) return "null server";
    std::lock_guard<std::mutex> lk(s->mu);
    return s->err.c_str();
}

extern "C" void pfg_server_destroy(pfg_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (std::thread& t : s->workers) t.join();
    for (pfg_ctx* c : s->ctx) pfg_destroy(c);
    delete s;
}
