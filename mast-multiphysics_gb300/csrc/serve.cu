// serve.cu -- the request loop (mg_server_*): continuous batching of SIMP design
// evaluations on one GPU.
//
// A worker thread owns the resident chains, held in a few shards (each one
// mg_batch with its chains' tables, solutions and multigrid hierarchy, on its
// own stream), and drives the multi-problem solver one graph launch (a few
// solver steps) at a time, the shards' launches running on the GPU together.
// Between launches it
//   * admits the requests that arrived: a request of a resident, idle chain gets
//     its densities and loads written and its load cases activated at the FP64
//     residual, warm-started from the chain's last solution, so it joins the
//     problems already in flight;
//   * admits new chains without stopping the others: when they fit under the
//     device-memory cap they get a shard of their own, or join a shard none of
//     whose chains is on the GPU when the shard count is at its limit;
//   * posts the requests whose load cases have all finished (compliance and
//     dC/drho written into the caller's buffers);
//   * only when the cap requires evictions (least recently used idle chains
//     first) does it let the in-flight work finish and rebuild one shard over
//     the retained and the new chains (keeping every retained chain's solutions).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

#include "batch.h"

namespace mg {
namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// MG_SERVER_TRACE=1: one line per worker event on stderr
bool trace_on() {
    static const bool on = getenv("MG_SERVER_TRACE") != nullptr;
    return on;
}
#define TRACE(...)                                        \
    do {                                                  \
        if (trace_on()) {                                 \
            fprintf(stderr, "[mg_server %.6f] ", now_s()); \
            fprintf(stderr, __VA_ARGS__);                 \
            fputc('\n', stderr);                          \
            fflush(stderr);                               \
        }                                                 \
    } while (0)

struct Request {
    mg_request r;
    std::vector<double> rho;
    std::vector<int32_t> span;
    double arrival = 0, admit = 0;
};

struct Chain {
    int id = 0;
    int nx = 0, ny = 0, nz = 0, n_cases = 0;
    int shard = -1;                  // resident shard (-1: not resident)
    int design = -1;                 // design index in that shard's batch
    bool rejected = false;           // does not fit the cap even alone
    bool has_solution = false;       // warm start available in the resident batch
    std::vector<int32_t> span;       // loads currently written into the batch
    std::vector<double> rho;         // densities of the last admitted request (host)
    std::deque<std::unique_ptr<Request>> queue;
    std::unique_ptr<Request> inflight;
    double last_used = 0;
    int64_t bytes = 0;               // estimated resident bytes
};

// resident bytes of one chain: every multigrid level of every load case
int64_t chain_bytes(int nx, int ny, int nz, int cases) {
    int64_t dofs = 0, elems = 0, nodes = 0;
    int x = nx, y = ny, z = nz;
    for (int lev = 0; lev < kMaxLevels; lev++) {
        const int64_t pitch = (3LL * (x + 1) + 3) / 4 * 4;
        dofs += pitch * (y + 1) * (z + 1);
        elems += (int64_t)((x + 3) / 4 * 4) * y * z;
        nodes += (int64_t)(x + 1) * (y + 1) * (z + 1);
        if (x % 2 || y % 2 || z % 2 || x < 4 || y < 4 || z < 4) break;
        x /= 2; y /= 2; z /= 2;
    }
    // 13 FP32 + 3 FP64 vectors per dof, 3 element tables per design, dc + densities
    return cases * (dofs * (13 * 4 + 3 * 8) + nodes + 8LL * nx * ny * nz) + elems * 20 +
           3 * 8LL * nx * ny * nz;
}

}  // namespace
}  // namespace mg

using namespace mg;

struct mg_server {
    int device = 0;                      // the creating thread's device
    mg_material_desc mat{};
    mg_server_opts opts{};
    std::thread worker;
    std::mutex mu;                       // inbox, completions, stats
    std::condition_variable cv_in, cv_out;
    std::deque<std::unique_ptr<Request>> inbox;
    std::deque<mg_completion> posted;
    std::vector<mg_completion> history;  // every completion (statistics)
    std::vector<int64_t> history_dofs;
    bool stop = false;
    int64_t submitted = 0, completed = 0, failed = 0, rebuilds = 0, evictions = 0;
    int64_t resident_bytes = 0, peak_resident = 0;
    int resident_chains = 0, inflight_now = 0, peak_inflight = 0;
    std::string worker_error;
    // worker-only state
    std::map<int, Chain> chains;
    std::vector<mg_batch *> shards;      // resident batches; the chains record theirs
};

namespace mg {
namespace {

void post(mg_server *s, const Request &q, int status, int its, int refs, double relres, int64_t dofs) {
    mg_completion c{};
    c.tag = q.r.tag;
    c.chain = q.r.chain;
    c.status = status;
    c.krylov_iterations = its;
    c.refinements = refs;
    c.relres = relres;
    c.arrival_s = q.arrival;
    c.admit_s = q.admit;
    c.done_s = now_s();
    std::lock_guard<std::mutex> lk(s->mu);
    s->posted.push_back(c);
    s->history.push_back(c);
    s->history_dofs.push_back(dofs);
    s->completed++;
    if (status != MG_OK) s->failed++;
    s->cv_out.notify_all();
}

constexpr int kMaxShards = 6;

void update_residency(mg_server *s) {
    int64_t bytes = 0;
    int n = 0;
    for (mg_batch *b : s->shards) bytes += b->device_bytes;
    for (auto &kv : s->chains) n += kv.second.shard >= 0 ? 1 : 0;
    std::lock_guard<std::mutex> lk(s->mu);
    s->resident_bytes = bytes;
    s->peak_resident = std::max(s->peak_resident, bytes);
    s->resident_chains = n;
}

// A new batch over the chains `order` (retained chains keep their solutions, copied
// from their current shards); the chains are pointed at it as shard `slot`, and the
// shards they came from are left to the caller.
int build_shard(mg_server *s, const std::vector<int> &order, int slot, mg_batch **out) {
    *out = nullptr;
    // stash the retained solutions (u of every load case) in one device buffer
    std::vector<std::pair<int, int64_t>> stash;  // (chain, offset)
    int64_t total = 0;
    for (int id : order) {
        Chain &c = s->chains[id];
        if (!c.has_solution || c.shard < 0) continue;
        mg_batch *old = s->shards[c.shard];
        stash.push_back({id, total});
        for (int k = 0; k < c.n_cases; k++) total += old->mf.h_probs[old->first[c.design] + k].n_pad;
    }
    double *d_stash = nullptr;
    if (total > 0) {
        MG_TRY(dev_alloc_n(&d_stash, (size_t)total));
        for (auto &st : stash) {
            Chain &c = s->chains[st.first];
            mg_batch *old = s->shards[c.shard];
            int64_t o = st.second;
            for (int k = 0; k < c.n_cases; k++) {
                const MfProblem &P = old->mf.h_probs[old->first[c.design] + k];
                cudaMemcpyAsync(d_stash + o, old->mf.u64 + P.dof_off, P.n_pad * 8, cudaMemcpyDeviceToDevice,
                                old->stream);
                o += P.n_pad;
            }
            cudaStreamSynchronize(old->stream);
        }
    }
    std::vector<mg_batch_problem> des(order.size());
    for (size_t i = 0; i < order.size(); i++) {
        Chain &c = s->chains[order[i]];
        // a new chain's first request provides its densities and loads
        const Request *q = c.queue.empty() ? nullptr : c.queue.front().get();
        if (c.rho.empty() && q) c.rho = q->rho;
        if (c.span.empty() && q) c.span = q->span;
        des[i].nx = c.nx;
        des[i].ny = c.ny;
        des[i].nz = c.nz;
        des[i].n_cases = c.n_cases;
        des[i].rho = c.rho.data();
        des[i].span = c.span.data();
    }
    mg_batch *nb = nullptr;
    int rc = mg_batch_create(des.data(), (int32_t)des.size(), &s->mat, &nb);
    if (rc != MG_OK) {
        dev_free(d_stash);
        return rc;
    }
    for (auto &st : stash) {
        Chain &c = s->chains[st.first];
        const int d = (int)(std::find(order.begin(), order.end(), st.first) - order.begin());
        int64_t o = st.second;
        for (int k = 0; k < c.n_cases; k++) {
            const MfProblem &P = nb->mf.h_probs[nb->first[d] + k];
            cudaMemcpyAsync(nb->mf.u64 + P.dof_off, d_stash + o, P.n_pad * 8, cudaMemcpyDeviceToDevice,
                            nb->stream);
            o += P.n_pad;
        }
    }
    cudaStreamSynchronize(nb->stream);
    dev_free(d_stash);
    rc = mf_batch_reset_states(nb->mf);
    if (rc == MG_OK) rc = mf_batch_prepare(nb->mf, params_from(s->opts.solve));
    if (rc != MG_OK) {
        mg_batch_destroy(nb);
        return rc;
    }
    for (size_t i = 0; i < order.size(); i++) {
        Chain &c = s->chains[order[i]];
        c.shard = slot;
        c.design = (int)i;
    }
    *out = nb;
    return MG_OK;
}

// every resident chain in `keep` plus the new chains `add` in one shard (the
// in-flight work has finished); the others are evicted
int rebuild_all(mg_server *s, const std::vector<int> &keep, const std::vector<int> &add) {
    TRACE("rebuild all: keep %zu add %zu", keep.size(), add.size());
    std::vector<int> order = keep;
    order.insert(order.end(), add.begin(), add.end());
    mg_batch *nb = nullptr;
    if (!order.empty()) MG_TRY(build_shard(s, order, 0, &nb));
    for (mg_batch *b : s->shards) mg_batch_destroy(b);
    s->shards.clear();
    for (auto &kv : s->chains)
        if (std::find(order.begin(), order.end(), kv.first) == order.end()) {
            kv.second.shard = -1;
            kv.second.design = -1;
        }
    if (nb) s->shards.push_back(nb);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->rebuilds++;  // every shard stopped for it
    }
    update_residency(s);
    return MG_OK;
}

// new chains that fit under the cap, without stopping the shards at work: a shard
// of their own, or, at the shard limit, a rebuild of a shard none of whose chains
// is on the GPU together with them; false when they have to wait
int admit_new(mg_server *s, const std::vector<int> &add, bool *admitted) {
    *admitted = false;
    if ((int)s->shards.size() < kMaxShards) {
        mg_batch *nb = nullptr;
        MG_TRY(build_shard(s, add, (int)s->shards.size(), &nb));
        s->shards.push_back(nb);
        TRACE("new shard %zu: %zu chains", s->shards.size() - 1, add.size());
        *admitted = true;
        update_residency(s);
        return MG_OK;
    }
    // the idle shard with the fewest chains
    int best = -1;
    size_t best_n = 0;
    for (int i = 0; i < (int)s->shards.size(); i++) {
        bool idle = true;
        size_t n = 0;
        for (auto &kv : s->chains)
            if (kv.second.shard == i) {
                n++;
                idle &= !kv.second.inflight;
            }
        if (idle && (best < 0 || n < best_n)) {
            best = i;
            best_n = n;
        }
    }
    if (best < 0) return MG_OK;  // every shard has work on the GPU: wait
    std::vector<int> order;
    for (auto &kv : s->chains)
        if (kv.second.shard == best) order.push_back(kv.first);
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        return s->chains[a].design < s->chains[b].design;
    });
    order.insert(order.end(), add.begin(), add.end());
    mg_batch *nb = nullptr;
    MG_TRY(build_shard(s, order, best, &nb));
    mg_batch_destroy(s->shards[best]);
    s->shards[best] = nb;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->rebuilds++;  // one idle shard rebuilt; the others kept working
    }
    TRACE("shard %d rebuilt with %zu new chains", best, add.size());
    *admitted = true;
    update_residency(s);
    return MG_OK;
}

// Admission plan for chains waiting to become resident (no side effects):
// waiting chains are taken in the order of their oldest pending request; each
// is admitted if it fits under the cap after evicting resident chains that are
// idle (least recently used first) or whose oldest pending request is younger
// than its own (youngest first).  The chain holding the oldest pending request
// of all can therefore always be admitted, and a chain that cannot be admitted
// does not hold back the resident chains' work.
struct AdmissionPlan {
    std::vector<int> keep, add, evict;
};

AdmissionPlan plan_admission(mg_server *s) {
    const int64_t cap = s->opts.hbm_cap_bytes > 0 ? s->opts.hbm_cap_bytes : (int64_t)150 << 30;
    AdmissionPlan pl;
    int64_t used = 0;
    for (auto &kv : s->chains)
        if (kv.second.shard >= 0) {
            pl.keep.push_back(kv.first);
            used += kv.second.bytes;
        }
    auto oldest = [&](const Chain &c) { return c.queue.empty() ? 1e300 : c.queue.front()->arrival; };
    std::vector<std::pair<double, int>> want;
    for (auto &kv : s->chains) {
        const Chain &c = kv.second;
        if (c.shard < 0 && !c.rejected && !c.queue.empty()) want.push_back({oldest(c), kv.first});
    }
    std::sort(want.begin(), want.end());
    for (auto &w : want) {
        const Chain &c = s->chains[w.second];
        if (c.bytes > cap) continue;  // answered with MG_ENOMEM by the caller
        std::vector<int> keep = pl.keep, evict;
        int64_t u = used;
        while (u + c.bytes > cap) {
            // idle chains: least recently used; busy ones: youngest pending request
            int idle_victim = -1, busy_victim = -1;
            double idle_lru = 1e300, busy_young = -1.0;
            for (int id : keep) {
                const Chain &v = s->chains[id];
                if (v.inflight) continue;
                if (v.queue.empty()) {
                    if (v.last_used < idle_lru) {
                        idle_lru = v.last_used;
                        idle_victim = id;
                    }
                } else if (oldest(v) > w.first && oldest(v) > busy_young) {
                    busy_young = oldest(v);
                    busy_victim = id;
                }
            }
            const int victim = idle_victim >= 0 ? idle_victim : busy_victim;
            if (victim < 0) break;
            keep.erase(std::find(keep.begin(), keep.end(), victim));
            evict.push_back(victim);
            u -= s->chains[victim].bytes;
        }
        if (u + c.bytes > cap) continue;  // waits; the resident chains keep working
        pl.keep = keep;
        pl.evict.insert(pl.evict.end(), evict.begin(), evict.end());
        pl.add.push_back(w.second);
        used = u + c.bytes;
    }
    return pl;
}

// answer the requests of chains that cannot fit even alone
void reject_oversized(mg_server *s) {
    const int64_t cap = s->opts.hbm_cap_bytes > 0 ? s->opts.hbm_cap_bytes : (int64_t)150 << 30;
    for (auto &kv : s->chains) {
        Chain &c = kv.second;
        if (c.shard < 0 && c.bytes > cap) c.rejected = true;
        while (c.rejected && !c.queue.empty()) {
            post(s, *c.queue.front(), MG_ENOMEM, 0, 0, 0.0, 0);
            c.queue.pop_front();
        }
    }
}

int apply_admission(mg_server *s, const AdmissionPlan &pl) {
    for (int id : pl.evict) {
        Chain &v = s->chains[id];
        v.has_solution = false;
        v.span.clear();
        std::lock_guard<std::mutex> lk(s->mu);
        s->evictions++;
    }
    return rebuild_all(s, pl.keep, pl.add);
}

// start the head request of an idle resident chain
int start_request(mg_server *s, Chain &c) {
    mg_batch *b = s->shards[c.shard];
    std::unique_ptr<Request> q = std::move(c.queue.front());
    c.queue.pop_front();
    q->admit = now_s();
    TRACE("start tag %llu chain %d design %d warm %d", (unsigned long long)q->r.tag, c.id, c.design,
          (int)c.has_solution);
    const int d = c.design;
    const int64_t ne = (int64_t)c.nx * c.ny * c.nz;
    MG_CUDA_TRY(cudaMemcpyAsync(b->d_rho + b->rho_off[d], q->rho.data(), ne * 8, cudaMemcpyHostToDevice,
                                b->stream));
    MG_TRY(refresh_moduli(b, d));
    if (q->span != c.span) {
        std::vector<uint8_t> fix;
        clamp_x0(c.nx, c.ny, c.nz, fix);
        std::vector<double> F;
        for (int k = 0; k < c.n_cases; k++) {
            line_load(c.nx, c.ny, c.nz, q->span[2 * k], q->span[2 * k + 1], F);
            MG_TRY(mf_batch_set_bc(b->mf, b->first[d] + k, fix.data(), F.data()));
        }
        c.span = q->span;
    }
    std::vector<int> probs;
    for (int k = 0; k < c.n_cases; k++) probs.push_back(b->first[d] + k);
    MG_TRY(mf_batch_activate(b->mf, probs, c.has_solution));
    MG_CUDA_TRY(cudaStreamSynchronize(b->stream));  // q->rho is a host buffer
    c.rho.swap(q->rho);
    c.inflight = std::move(q);
    return MG_OK;
}

// post the finished requests (chains of shard b)
int finish_requests(mg_server *s, mg_batch *b, const std::vector<int> &done_chains) {
    std::vector<uint8_t> active(b->n_probs, 0);
    for (int id : done_chains) {
        Chain &c = s->chains[id];
        for (int k = 0; k < c.n_cases; k++) {
            const int i = b->first[c.design] + k;
            mf_batch_finish(b->mf, i);
            active[i] = 1;
        }
    }
    MG_TRY(batch_results_of(b, active.data()));
    for (int id : done_chains) {
        Chain &c = s->chains[id];
        Request &q = *c.inflight;
        const int64_t ne = (int64_t)c.nx * c.ny * c.nz;
        int status = MG_OK, its = 0, refs = 0;
        double relres = 0.0;
        for (int k = 0; k < c.n_cases; k++) {
            const int i = b->first[c.design] + k;
            const mg_solve_report &r = b->reports[i];
            if (r.status != MG_OK && status == MG_OK) status = r.status;
            its += r.krylov_iterations;
            refs = std::max(refs, r.refinements);
            relres = std::max(relres, r.relres);
            if (q.r.compliance_out) q.r.compliance_out[k] = b->compliance[i];
            if (q.r.dc_out)
                MG_CUDA_TRY(cudaMemcpyAsync(q.r.dc_out + k * ne, b->d_dc + b->dc_off[i], ne * 8,
                                            cudaMemcpyDeviceToHost, b->stream));
        }
        MG_CUDA_TRY(cudaStreamSynchronize(b->stream));
        c.has_solution = (status == MG_OK);
        c.last_used = now_s();
        std::unique_ptr<Request> done = std::move(c.inflight);
        TRACE("done tag %llu chain %d status %d its %d relres %.2e", (unsigned long long)done->r.tag, c.id,
              status, its, relres);
        post(s, *done, status, its, refs, relres, c.n_cases * dofs_of(c.nx, c.ny, c.nz));
    }
    return MG_OK;
}

void worker_main(mg_server *s) {
    cudaSetDevice(s->device);
    auto fail_all = [&](int rc) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->worker_error = mg_last_error();
        }
        for (auto &kv : s->chains) {
            Chain &c = kv.second;
            if (c.inflight) post(s, *c.inflight, rc, 0, 0, 0.0, 0);
            c.inflight.reset();
            while (!c.queue.empty()) {
                post(s, *c.queue.front(), rc, 0, 0, 0.0, 0);
                c.queue.pop_front();
            }
        }
    };
    for (;;) {
        bool stopping = false;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            const bool busy = s->inflight_now > 0;
            bool pending = false;
            for (auto &kv : s->chains) pending |= !kv.second.queue.empty();
            if (!busy && !pending && s->inbox.empty() && !s->stop)
                s->cv_in.wait_for(lk, std::chrono::milliseconds(2));
            while (!s->inbox.empty()) {
                std::unique_ptr<Request> q = std::move(s->inbox.front());
                s->inbox.pop_front();
                Chain &c = s->chains[q->r.chain];
                if (c.n_cases == 0) {
                    c.id = q->r.chain;
                    c.nx = q->r.nx; c.ny = q->r.ny; c.nz = q->r.nz; c.n_cases = q->r.n_cases;
                    c.bytes = chain_bytes(c.nx, c.ny, c.nz, c.n_cases);
                }
                if (c.nx != q->r.nx || c.ny != q->r.ny || c.nz != q->r.nz || c.n_cases != q->r.n_cases) {
                    lk.unlock();
                    post(s, *q, MG_EINVAL, 0, 0, 0.0, 0);  // contradicts its chain
                    lk.lock();
                    continue;
                }
                c.queue.push_back(std::move(q));
            }
            stopping = s->stop;
        }
        int rc = MG_OK;
        reject_oversized(s);
        // new chains: admitted at once when they fit under the cap (a shard of their
        // own); when the cap requires evictions, admissions of resident chains pause
        // until the in-flight work has finished and one shard is rebuilt
        bool waiting = false;
        for (auto &kv : s->chains)
            waiting |= (kv.second.shard < 0 && !kv.second.rejected && !kv.second.queue.empty());
        AdmissionPlan plan;
        if (waiting) plan = plan_admission(s);
        int inflight = 0;
        for (auto &kv : s->chains) inflight += kv.second.inflight ? 1 : 0;
        bool need_rebuild = false;
        if (!plan.add.empty()) {
            if (plan.evict.empty()) {
                bool admitted = false;
                rc = admit_new(s, plan.add, &admitted);
            } else {
                need_rebuild = true;
                if (inflight == 0) rc = apply_admission(s, plan);
            }
        }
        // admit requests of resident idle chains unless a rebuild is waiting
        if (rc == MG_OK && !need_rebuild && !s->shards.empty()) {
            const int cap = s->opts.max_inflight > 0 ? s->opts.max_inflight : 1 << 30;
            std::vector<std::pair<double, int>> ready;
            for (auto &kv : s->chains) {
                Chain &c = kv.second;
                if (c.shard >= 0 && !c.inflight && !c.queue.empty()) ready.push_back({c.queue.front()->arrival, kv.first});
            }
            std::sort(ready.begin(), ready.end());
            for (auto &r : ready) {
                if (inflight >= cap) break;
                rc = start_request(s, s->chains[r.second]);
                if (rc != MG_OK) break;
                inflight++;
            }
        }
        // watchdog: a request on the GPU longer than the solve's wall-clock limit
        // is answered with MG_ETIMEDOUT and its load cases are stopped
        if (rc == MG_OK && inflight > 0) {
            const double limit = s->opts.solve.timeout_s > 0 ? s->opts.solve.timeout_s : 600.0;
            const double now = now_s();
            for (auto &kv : s->chains) {
                Chain &c = kv.second;
                if (!c.inflight || now - c.inflight->admit <= limit) continue;
                mg_batch *b = s->shards[c.shard];
                for (int k = 0; k < c.n_cases; k++) {
                    const int i = b->first[c.design] + k;
                    MfState &h = b->mf.states_host[i];
                    h.phase = kPhaseFin;
                    h.done = 1;
                    h.ref_done = 1;
                    rc = cudaMemcpyAsync(b->mf.states + i, &h, sizeof(MfState), cudaMemcpyHostToDevice, b->stream)
                             == cudaSuccess ? MG_OK : MG_ECUDA;
                }
                cudaStreamSynchronize(b->stream);
                c.has_solution = false;
                std::unique_ptr<Request> q = std::move(c.inflight);
                post(s, *q, MG_ETIMEDOUT, 0, 0, 0.0, 0);
                inflight--;
            }
        }
        if (rc == MG_OK && inflight > 0) {
            // one graph launch on every shard with work, all on the GPU at once
            std::vector<int> busy(s->shards.size(), 0);
            for (auto &kv : s->chains)
                if (kv.second.inflight) busy[kv.second.shard] = 1;
            for (size_t i = 0; i < s->shards.size() && rc == MG_OK; i++)
                if (busy[i]) rc = mf_batch_step_begin(s->shards[i]->mf);
            for (size_t i = 0; i < s->shards.size(); i++)
                if (busy[i]) {
                    const int r2 = mf_batch_step_end(s->shards[i]->mf);
                    if (rc == MG_OK) rc = r2;
                }
            for (size_t i = 0; i < s->shards.size() && rc == MG_OK; i++) {
                if (!busy[i]) continue;
                mg_batch *b = s->shards[i];
                std::vector<int> done;
                for (auto &kv : s->chains) {
                    Chain &c = kv.second;
                    if (!c.inflight || c.shard != (int)i) continue;
                    bool fin = true;
                    for (int k = 0; k < c.n_cases; k++) fin &= b->mf.states_host[b->first[c.design] + k].phase == kPhaseFin;
                    if (fin) done.push_back(kv.first);
                }
                if (!done.empty()) rc = finish_requests(s, b, done);
                inflight -= (int)done.size();
            }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->inflight_now = inflight;
            s->peak_inflight = std::max(s->peak_inflight, inflight);
        }
        if (rc != MG_OK) {
            TRACE("error %d: %s", rc, mg_last_error());
            // answer everything with the error and start again from no resident chain
            fail_all(rc);
            for (mg_batch *b : s->shards) mg_batch_destroy(b);
            s->shards.clear();
            for (auto &kv : s->chains) {
                kv.second.shard = -1;
                kv.second.design = -1;
                kv.second.has_solution = false;
                kv.second.span.clear();
            }
            std::lock_guard<std::mutex> lk(s->mu);
            s->inflight_now = 0;
            s->resident_chains = 0;
            s->resident_bytes = 0;
        }
        if (stopping) {
            std::lock_guard<std::mutex> lk(s->mu);
            bool pending = !s->inbox.empty() || s->inflight_now > 0;
            for (auto &kv : s->chains) pending |= !kv.second.queue.empty();
            if (!pending) break;
        }
        if (inflight == 0 && !(need_rebuild && rc == MG_OK)) {
            // nothing on the GPU and nothing admitted: wait for a submission
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->inbox.empty() && !s->stop) s->cv_in.wait_for(lk, std::chrono::milliseconds(1));
        }
    }
    for (mg_batch *b : s->shards) mg_batch_destroy(b);
    s->shards.clear();
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double x = p * (v.size() - 1);
    const size_t i = (size_t)x;
    const double f = x - i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

void stats_of(const std::vector<mg_completion> &h, const std::vector<int64_t> &dofs, size_t lo,
              mg_server_stats *out) {
    std::vector<double> lat;
    double first = 1e300, last = 0.0;
    int64_t ndofs = 0, ok = 0;
    for (size_t i = lo; i < h.size(); i++) {
        if (h[i].status != MG_OK) continue;
        lat.push_back(h[i].done_s - h[i].arrival_s);
        first = std::min(first, h[i].arrival_s);
        last = std::max(last, h[i].done_s);
        ndofs += dofs[i];
        ok++;
    }
    out->p50_s = percentile(lat, 0.50);
    out->p99_s = percentile(lat, 0.99);
    double sum = 0, mx = 0;
    for (double x : lat) {
        sum += x;
        mx = std::max(mx, x);
    }
    out->mean_s = lat.empty() ? 0.0 : sum / lat.size();
    out->max_s = mx;
    const double span = last - first;
    out->solves_per_s = (ok > 0 && span > 0) ? ok / span : 0.0;
    out->dofs_per_s = (ok > 0 && span > 0) ? ndofs / span : 0.0;
}

bool request_ok(const mg_request &r) {
    if (r.chain < 0 || r.nx <= 0 || r.ny <= 0 || r.nz <= 0 || r.nx > 4096 || r.ny > 4096 || r.nz > 4096)
        return false;
    if (r.n_cases < 1 || r.n_cases > MG_BATCH_MAX_CASES || !r.rho || !r.span) return false;
    for (int k = 0; k < r.n_cases; k++)
        if (r.span[2 * k] < 0 || r.span[2 * k] > r.span[2 * k + 1] || r.span[2 * k + 1] > r.ny) return false;
    const int64_t ne = (int64_t)r.nx * r.ny * r.nz;
    for (int64_t e = 0; e < ne; e++)
        if (!(r.rho[e] >= 0.0 && r.rho[e] <= 1.0)) return false;
    return true;
}

}  // namespace
}  // namespace mg

extern "C" {

double mg_server_clock(void) { return now_s(); }

int mg_server_create(const mg_material_desc *mat, const mg_server_opts *opts, mg_server **out) {
    if (!out) return MG_EINVAL;
    *out = nullptr;
    if (!mat || !opts || !material_ok(*mat)) {
        set_error("mg_server_create: bad material or options");
        return MG_EINVAL;
    }
    if (opts->solve.precision < MG_MIXED_TF32 || opts->solve.precision > MG_MIXED_BF16X3) {
        set_error("the request loop serves the mixed-precision forms");
        return MG_ENOTSUP;
    }
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return MG_ECUDA;
    }
    mg_server *s = new mg_server();
    cudaGetDevice(&s->device);
    s->mat = *mat;
    s->opts = *opts;
    s->worker = std::thread(worker_main, s);
    *out = s;
    return MG_OK;
}

int mg_server_submit(mg_server *s, const mg_request *req) {
    if (!s || !req || !request_ok(*req)) {
        set_error("malformed request");
        return MG_EINVAL;
    }
    std::unique_ptr<Request> q(new Request());
    q->r = *req;
    const int64_t ne = (int64_t)req->nx * req->ny * req->nz;
    q->rho.assign(req->rho, req->rho + ne);
    q->span.assign(req->span, req->span + 2 * req->n_cases);
    q->arrival = req->arrival_s > 0 ? req->arrival_s : now_s();
    q->r.rho = nullptr;
    q->r.span = nullptr;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        set_error("server is shutting down");
        return MG_EBUSY;
    }
    // a chain keeps its grid and number of load cases
    for (auto &p : s->inbox)
        if (p->r.chain == req->chain && (p->r.nx != req->nx || p->r.ny != req->ny || p->r.nz != req->nz ||
                                          p->r.n_cases != req->n_cases)) {
            set_error("request contradicts chain %d", req->chain);
            return MG_EINVAL;
        }
    s->inbox.push_back(std::move(q));
    s->submitted++;
    s->cv_in.notify_one();
    return MG_OK;
}

int mg_server_poll(mg_server *s, mg_completion *out, int32_t max, int32_t *n, double timeout_s) {
    if (!s || !n || (max > 0 && !out)) return MG_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->posted.empty() && timeout_s > 0)
        s->cv_out.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return !s->posted.empty(); });
    int k = 0;
    while (k < max && !s->posted.empty()) {
        out[k++] = s->posted.front();
        s->posted.pop_front();
    }
    *n = k;
    return MG_OK;
}

int mg_server_drain(mg_server *s, double timeout_s) {
    if (!s) return MG_EINVAL;
    const double t0 = now_s();
    std::unique_lock<std::mutex> lk(s->mu);
    while (s->completed < s->submitted) {
        s->cv_out.wait_for(lk, std::chrono::milliseconds(50));
        if (timeout_s > 0 && now_s() - t0 > timeout_s) {
            set_error("drain: %lld of %lld requests still open", (long long)(s->submitted - s->completed),
                      (long long)s->submitted);
            return MG_ETIMEDOUT;
        }
    }
    return MG_OK;
}

int mg_server_get_stats(mg_server *s, mg_server_stats *out) {
    if (!s || !out) return MG_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->rebuilds = s->rebuilds;
    out->evictions = s->evictions;
    out->resident_bytes = s->resident_bytes;
    out->peak_resident_bytes = s->peak_resident;
    out->resident_chains = s->resident_chains;
    out->inflight = s->inflight_now;
    out->peak_inflight = s->peak_inflight;
    stats_of(s->history, s->history_dofs, 0, out);
    return MG_OK;
}

void mg_server_destroy(mg_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_in.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    delete s;
}

}  // extern "C"

namespace {
// The synthetic stream: chain grids, load cases and spans, arrival times and the chain
// of every request, all from one seeded generator (cheap); densities come per chain.
struct SynthChain {
    int nx, ny, nz, cases;
    std::vector<int32_t> span;
};

struct SynthStream {
    std::vector<SynthChain> ch;
    std::vector<double> at;
    std::vector<int> who;
};

bool synth_valid(const mg_synthetic_desc *d) {
    return d && d->n_requests > 0 && d->rate > 0 && d->n_chains > 0 && d->n_sizes > 0 && d->sizes &&
           d->max_cases >= 1 && d->max_cases <= MG_BATCH_MAX_CASES;
}

void synth_stream(const mg_synthetic_desc *d, SynthStream &st) {
    const int nch = d->n_chains;
    std::mt19937_64 rng(d->seed);
    st.ch.assign(nch, SynthChain{});
    int n_big = d->big_fraction > 0 ? std::max(1, (int)lround(d->big_fraction * nch)) : 0;
    for (int c = 0; c < nch; c++) {
        SynthChain &g = st.ch[c];
        if (c < n_big) {
            g.nx = d->big_nx; g.ny = d->big_ny; g.nz = d->big_nz;
        } else {
            const int k = (int)(rng() % (uint64_t)d->n_sizes);
            g.nx = d->sizes[3 * k]; g.ny = d->sizes[3 * k + 1]; g.nz = d->sizes[3 * k + 2];
        }
        g.cases = 1 + (int)(rng() % (uint64_t)d->max_cases);
        for (int k = 0; k < g.cases; k++) {
            const int j0 = (int)(rng() % (uint64_t)(g.ny + 1));
            const int j1 = j0 + (int)(rng() % (uint64_t)(g.ny + 1 - j0));
            g.span.push_back(j0);
            g.span.push_back(j1);
        }
    }
    st.at.assign(d->n_requests, 0.0);
    st.who.assign(d->n_requests, 0);
    std::exponential_distribution<double> gap(d->rate);
    double t = 0;
    for (int64_t i = 0; i < d->n_requests; i++) {
        t += gap(rng);
        st.at[i] = t;
        st.who[i] = (int)(rng() % (uint64_t)nch);
    }
}

// Walks chain c's density field through the chain's requests in index order
// (rho_next = clip(rho + N(0, noise), 0.01, 1) per request, from a U[0.01, 1] start);
// emit(i, field) is called with the field of each request i of the chain.
template <class F>
void synth_chain_fields(const mg_synthetic_desc *d, const SynthStream &st, int c,
                        const std::vector<int64_t> &requests, F emit) {
    const SynthChain &g = st.ch[c];
    const int64_t ne = (int64_t)g.nx * g.ny * g.nz;
    std::mt19937_64 r2(d->seed * 1000003ULL + (uint64_t)c + 1);
    std::uniform_real_distribution<float> U(0.01f, 1.0f);
    std::normal_distribution<float> N(0.0f, (float)d->noise);
    std::vector<float> cur(ne);
    for (auto &x : cur) x = U(r2);
    for (int64_t i : requests) {
        for (auto &x : cur) x = std::min(1.0f, std::max(0.01f, x + N(r2)));
        if (!emit(i, cur)) return;
    }
}
}  // namespace

extern "C" {

int mg_server_synthetic_request(const mg_synthetic_desc *d, int64_t index, int32_t *info,
                                int32_t *span, double *rho) {
    if (!synth_valid(d) || index < 0 || index >= d->n_requests || !info) {
        set_error("mg_server_synthetic_request: invalid argument");
        return MG_EINVAL;
    }
    SynthStream st;
    synth_stream(d, st);
    const int c = st.who[index];
    const SynthChain &g = st.ch[c];
    info[0] = c;
    info[1] = g.nx;
    info[2] = g.ny;
    info[3] = g.nz;
    info[4] = g.cases;
    if (span)
        for (int k = 0; k < 2 * g.cases; k++) span[k] = g.span[k];
    if (rho) {
        std::vector<int64_t> req;
        for (int64_t i = 0; i <= index; i++)
            if (st.who[i] == c) req.push_back(i);
        synth_chain_fields(d, st, c, req, [&](int64_t i, const std::vector<float> &f) {
            if (i != index) return true;
            for (size_t k = 0; k < f.size(); k++) rho[k] = (double)f[k];
            return false;
        });
    }
    return MG_OK;
}

int mg_server_run_synthetic(mg_server *s, const mg_synthetic_desc *d, double *compliance_out,
                            mg_server_stats *stats) {
    if (!s || !synth_valid(d)) return MG_EINVAL;
    const int nch = d->n_chains;
    SynthStream ss;
    synth_stream(d, ss);
    const std::vector<SynthChain> &ch = ss.ch;
    const std::vector<double> &at = ss.at;
    const std::vector<int> &who = ss.who;
    // densities of every request, chain by chain (threads over chains)
    std::vector<std::vector<float>> fields(d->n_requests);
    {
        std::vector<std::vector<int64_t>> per(nch);
        for (int64_t i = 0; i < d->n_requests; i++) per[who[i]].push_back(i);
        const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (unsigned w = 0; w < nt; w++)
            th.emplace_back([&, w] {
                for (int c = (int)w; c < nch; c += (int)nt)
                    synth_chain_fields(d, ss, c, per[c], [&](int64_t i, const std::vector<float> &f) {
                        fields[i] = f;
                        return true;
                    });
            });
        for (auto &x : th) x.join();
    }
    size_t h0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        h0 = s->history.size();
    }
    std::vector<double> comp((size_t)d->n_requests * d->max_cases, 0.0);
    // submit at the arrival times (the densities are converted to FP64 per request)
    const double t0 = now_s() + 0.05;
    int rc = MG_OK;
    for (int64_t i = 0; i < d->n_requests && rc == MG_OK; i++) {
        const SynthChain &g = ch[who[i]];
        std::vector<double> rho(fields[i].begin(), fields[i].end());
        std::vector<float>().swap(fields[i]);
        mg_request q{};
        q.chain = who[i];
        q.nx = g.nx; q.ny = g.ny; q.nz = g.nz;
        q.n_cases = g.cases;
        q.rho = rho.data();
        q.span = g.span.data();
        q.compliance_out = comp.data() + i * d->max_cases;
        q.arrival_s = t0 + at[i];
        q.tag = (uint64_t)i;
        while (now_s() < q.arrival_s) {
            const double w = q.arrival_s - now_s();
            if (w > 2e-3) std::this_thread::sleep_for(std::chrono::duration<double>(w - 1e-3));
        }
        rc = mg_server_submit(s, &q);
    }
    if (rc == MG_OK) rc = mg_server_drain(s, 0.0);
    if (compliance_out) memcpy(compliance_out, comp.data(), comp.size() * sizeof(double));
    if (stats) {
        std::lock_guard<std::mutex> lk(s->mu);
        memset(stats, 0, sizeof(*stats));
        stats->submitted = d->n_requests;
        for (size_t i = h0; i < s->history.size(); i++) {
            stats->completed++;
            if (s->history[i].status != MG_OK) stats->failed++;
        }
        stats->rebuilds = s->rebuilds;
        stats->evictions = s->evictions;
        stats->resident_bytes = s->resident_bytes;
        stats->peak_resident_bytes = s->peak_resident;
        stats->resident_chains = s->resident_chains;
        stats->peak_inflight = s->peak_inflight;
        stats_of(s->history, s->history_dofs, h0, stats);
    }
    return rc;
}

}  // extern "C"
