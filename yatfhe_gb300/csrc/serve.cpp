// serve.cpp -- multi-tenant bootstrap serving with continuous batching and an HBM key cache.
//
// Semantics follow the reference's CPU serving harness (ya_benchmark/blindrotate_serving.cpp,
// ya_benchmark/include/blindrotate_serving.h): requests (tenant, ciphertexts) arrive as a
// Poisson process (ArrivalProcess, blindrotate_serving.h:309-350; generator mt19937_64 seeded
// with seed ^ 0x9e3779b97f4a7c15, blindrotate_serving.cpp:184), tenants are Zipf-popular
// (ZipfDistribution, yatfhe/include/yautil/zipf.h:47-87), keys live in an LRU cache
// (ConcurrentKeyCache, blindrotate_serving.h:25-111) and latency is reported as ceil-rank
// percentiles of sojourn / queue / service time (blindrotate_serving.cpp:60-82).
//
// GPU design.  One worker thread owns the device.  Tenant keys are kept, already in the
// device layout, in pinned host memory; HBM holds `slots` of them (budget / key bytes),
// refilled on a miss by cudaMemcpyAsync on a copy stream, with an event the batch's stream
// waits on.  The worker admits pending requests into a batch (up to max_batch ciphertexts),
// in arrival order, as long as their keys are resident or can be brought in (an LRU slot
// whose tenant has no batch in flight); a request larger than what is left of the batch is
// split, its first part filling the batch and the rest opening the next one, so batches
// leave the worker full whenever enough work is queued.  The batch is grouped by tenant and
// the multi-key blind rotation and key switch are launched.  Up to max_inflight batches are on the GPU at once, each on its own
// stream, so requests that arrive while one runs are admitted into the next (continuous
// batching) and the next batch fills the SMs the previous one's last wave leaves idle.
// Batch completion is signalled by a host callback on the batch's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.hpp"

namespace {

using Clock = std::chrono::steady_clock;
using yg::ck;
using yg::guarded;
using yg::set_err;

double now_s() { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); }

struct Request {
    int64_t id = 0;
    int tenant = 0;
    int count = 0;
    const int32_t* h_in = nullptr;
    int32_t* h_out = nullptr;
    double t_submit = 0, t_start = 0, t_done = 0;
    int admitted = 0;    // ciphertexts placed in batches so far
    int parts_open = 0;  // placed parts whose batch has not retired
    std::atomic<bool> done{false};
};

// A contiguous part of a request inside one batch.
struct Part {
    Request* r;
    int offset, count;
};

// Smallest part a request is split into to fill a batch (smaller rests close the batch).
constexpr int kMinPart = 16;

struct Tenant {
    int id = 0;
    int index = 0;                 // dense index (LUT table)
    uint32_t* h_bsk = nullptr;     // pinned, device layout
    int32_t* h_ksk = nullptr;      // pinned
    int64_t* d_lut = nullptr;
    int slot = -1;
    cudaEvent_t ready = nullptr;
    int pins = 0;
    uint64_t last_use = 0;
};

struct Batch {
    cudaStream_t stream = nullptr;  // batches in flight run on their own streams and overlap
    int32_t* d_in = nullptr;
    int32_t* d_out = nullptr;
    int32_t* d_big = nullptr;
    int32_t* d_key_of = nullptr;
    int32_t* d_lut_of = nullptr;
    yg::KsTile* d_tiles = nullptr;
    int32_t* h_key_of = nullptr;   // pinned staging
    int32_t* h_lut_of = nullptr;
    yg::KsTile* h_tiles = nullptr;
    std::vector<Part> parts;
    std::vector<Tenant*> tenants;
    double t_finish = 0;  // stamped by the completion callback
    int refills = 0;      // key refills this batch issued (in flight until it retires)
    std::atomic<bool> finished{false};
    bool busy = false;
    struct yg_server* server = nullptr;
};

}  // namespace

struct yg_server {
    yg_ctx* ctx = nullptr;
    yg_server_config cfg{};
    size_t bsk_bytes = 0, ksk_bytes = 0;
    // The key family of the tenants, fixed by the first one: GINX rows (and keys derived into
    // them), or lazy keys, whose slot holds [half rows | table block] and whose batches run
    // the lazy blind rotation with a per-slot key table and server-owned transform tables.
    bool family_set = false, lazy = false;
    int lazy_ls = 0;
    size_t lazy_cprime_bytes = 0;
    yg::LazyBrArgs lazy_tmpl{};
    yg::LazyKeyRef* d_lazy_slot_table = nullptr;
    uint64_t* d_lazy_tables = nullptr;
    int nslots = 0;
    std::vector<uint32_t*> slot_bsk;
    std::vector<int32_t*> slot_ksk;
    std::vector<int> slot_owner;
    const uint4** d_slot_table = nullptr;
    const int64_t** d_lut_table = nullptr;
    std::map<int, std::unique_ptr<Tenant>> tenants;
    std::vector<Tenant*> by_index;
    cudaStream_t copy = nullptr;
    std::vector<std::unique_ptr<Batch>> batches;

    std::mutex mu;
    std::condition_variable cv;        // worker wake-ups (arrivals, batch completion)
    std::condition_variable cv_done;   // waiters in yg_server_wait
    std::deque<Request*> incoming;
    std::unordered_map<int64_t, std::unique_ptr<Request>> requests;
    int64_t next_id = 1;
    std::thread worker;
    bool running = false, stopping = false;
    uint64_t tick = 0;
    std::string worker_error;

    // statistics
    uint64_t hits = 0, misses = 0, refill_bytes = 0, batches_run = 0, ciphertexts_done = 0, requests_done = 0;
    // GINX batches of at most latency_max ciphertexts run in the channel-cluster layout
    int latency_max = 0;
    uint64_t latency_batches_run = 0;
    // requests submitted and not yet started (the reference's queue depth, peak since the
    // last reset); key refills of batches not yet retired, sampled at every launch
    int waiting = 0, waiting_peak = 0;
    int refills_inflight = 0, refills_peak = 0;
    uint64_t refill_samples = 0, refill_sample_sum = 0;
    double busy_since = 0;
};

namespace {

// Host callback at the end of a batch.  It runs on a CUDA thread and must not take the
// server lock (the worker holds it across CUDA calls), so it only stamps and flags; the
// worker's timed wait picks the flag up.
void CUDART_CB batch_done_cb(void* p) {
    Batch* b = static_cast<Batch*>(p);
    b->t_finish = now_s();
    b->finished.store(true);
    b->server->cv.notify_all();
}

void free_batch(Batch* b) {
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->stream) cudaStreamDestroy(b->stream);
    cudaFree(b->d_in);
    cudaFree(b->d_out);
    cudaFree(b->d_big);
    cudaFree(b->d_key_of);
    cudaFree(b->d_lut_of);
    cudaFree(b->d_tiles);
    cudaFreeHost(b->h_key_of);
    cudaFreeHost(b->h_lut_of);
    cudaFreeHost(b->h_tiles);
}

// Retires finished batches (caller holds the lock).
void retire(yg_server* s) {
    for (auto& bp : s->batches) {
        Batch* b = bp.get();
        if (!b->busy || !b->finished.load()) continue;
        for (const Part& part : b->parts) {
            Request* r = part.r;
            r->t_done = std::max(r->t_done, b->t_finish);
            s->ciphertexts_done += part.count;
            if (--r->parts_open == 0 && r->admitted == r->count) {
                r->done.store(true);
                s->requests_done++;
            }
        }
        for (Tenant* t : b->tenants) t->pins--;
        s->refills_inflight -= b->refills;
        b->refills = 0;
        b->parts.clear();
        b->tenants.clear();
        b->busy = false;
        b->finished.store(false);
    }
    s->cv_done.notify_all();
}

// A slot for tenant t: free, or the least recently used whose tenant has nothing in
// flight and is not in the batch being formed (pins == 0).  -1 if none.
int find_slot(yg_server* s) {
    int best = -1;
    uint64_t best_use = UINT64_MAX;
    for (int i = 0; i < s->nslots; i++) {
        const int owner = s->slot_owner[i];
        if (owner < 0) return i;
        Tenant* o = s->tenants[owner].get();
        if (o->pins == 0 && o->last_use < best_use) {
            best = i;
            best_use = o->last_use;
        }
    }
    return best;
}

// Builds and launches one batch from the pending queue (caller holds the lock).
bool launch_batch(yg_server* s, std::deque<Request*>& pending, Batch* b) {
    const yg_params& p = s->ctx->p;
    const int n1 = p.n + 1, kN = p.k * p.N;
    int total = 0;
    std::vector<Part> take;
    std::vector<Tenant*> used;
    int refills = 0;
    while (!pending.empty()) {
        Request* r = pending.front();
        const int rest = r->count - r->admitted, room = s->cfg.max_batch - total;
        if (room <= 0 || (rest > room && room < kMinPart && total > 0)) break;
        const int part = std::min(rest, room);
        Tenant* t = s->tenants[r->tenant].get();
        const bool in_batch = std::find(used.begin(), used.end(), t) != used.end();
        if (t->slot < 0) {
            const int slot = find_slot(s);
            if (slot < 0) break;  // every slot is held by work in flight: admit later
            const int prev = s->slot_owner[slot];
            if (prev >= 0) s->tenants[prev]->slot = -1;
            s->slot_owner[slot] = t->id;
            t->slot = slot;
            ck(cudaMemcpyAsync(s->slot_bsk[slot], t->h_bsk, s->bsk_bytes, cudaMemcpyHostToDevice, s->copy), "refill");
            ck(cudaMemcpyAsync(s->slot_ksk[slot], t->h_ksk, s->ksk_bytes, cudaMemcpyHostToDevice, s->copy), "refill");
            ck(cudaEventRecord(t->ready, s->copy), "refill event");
            s->misses++;
            s->refill_bytes += s->bsk_bytes + s->ksk_bytes;
            refills++;
        } else if (!in_batch) {
            s->hits++;
        }
        if (!in_batch) {
            used.push_back(t);
            t->pins++;  // from here on the slot cannot be taken by another tenant
        }
        t->last_use = ++s->tick;
        take.push_back(Part{r, r->admitted, part});
        r->admitted += part;
        r->parts_open++;
        total += part;
        if (r->admitted < r->count) break;  // the batch is full; the rest opens the next one
        pending.pop_front();
    }
    if (take.empty()) return false;
    // group by tenant so the key switch streams one KSK per run of ciphertexts
    std::stable_sort(take.begin(), take.end(), [](const Part& a, const Part& b) { return a.r->tenant < b.r->tenant; });
    const double t0 = now_s();
    int off = 0, ntiles = 0;
    for (const Part& part : take) {
        Request* r = part.r;
        Tenant* t = s->tenants[r->tenant].get();
        if (part.offset == 0) {
            r->t_start = t0;
            s->waiting--;
        }
        ck(cudaMemcpyAsync(b->d_in + (size_t)off * n1, r->h_in + (size_t)part.offset * n1, (size_t)part.count * n1 * 4,
                           cudaMemcpyHostToDevice, b->stream),
           "copy in");
        for (int c = 0; c < part.count; c++) {
            b->h_key_of[off + c] = t->slot;
            b->h_lut_of[off + c] = t->index;
        }
        off += part.count;
    }
    for (int c = 0; c < total;) {
        int e = c + 1;
        while (e < total && e - c < yg::kKsTileCts && b->h_key_of[e] == b->h_key_of[c]) e++;
        b->h_tiles[ntiles++] = yg::KsTile{c, e - c, s->slot_ksk[b->h_key_of[c]]};
        c = e;
    }
    ck(cudaMemcpyAsync(b->d_key_of, b->h_key_of, (size_t)total * 4, cudaMemcpyHostToDevice, b->stream), "tables");
    ck(cudaMemcpyAsync(b->d_lut_of, b->h_lut_of, (size_t)total * 4, cudaMemcpyHostToDevice, b->stream), "tables");
    ck(cudaMemcpyAsync(b->d_tiles, b->h_tiles, (size_t)ntiles * sizeof(yg::KsTile), cudaMemcpyHostToDevice, b->stream),
       "tables");
    for (Tenant* t : used) ck(cudaStreamWaitEvent(b->stream, t->ready, 0), "wait refill");
    if (s->lazy) {
        yg::LazyBrArgs la = s->lazy_tmpl;
        la.keys = s->d_lazy_slot_table;
        la.key_of = b->d_key_of;
        la.lut_table = s->d_lut_table;
        la.lut_of = b->d_lut_of;
        la.lwe_in = b->d_in;
        la.big_out = b->d_big;
        la.count = total;
        yg::check_launch(yg::launch_lazy_blind_rotate(la, b->stream), "lazy blind rotate launch");
    } else {
    yg::BrArgs a = yg::br_args(s->ctx, nullptr);
    a.key = nullptr;
    a.key_table = s->d_slot_table;
    a.key_of = b->d_key_of;
    a.lut_table = s->d_lut_table;
    a.lut_of = b->d_lut_of;
    a.lwe_in = b->d_in;
    a.big_out = b->d_big;
    a.count = total;
    if (total <= s->latency_max) {
        a.layout = yg::kLayoutChannelCluster;
        a.per_cta = 1;
        a.grid = 0;
        s->latency_batches_run++;
    }
    yg::check_launch(yg::launch_blind_rotate(s->ctx->logN, p.torus_bits, a, b->stream), "blind rotate launch");
    }
    yg::KsArgs k{b->d_big, nullptr, b->d_out, total, kN, p.n, p.ks_level, p.ks_radix_bits, b->d_tiles, ntiles};
    yg::check_launch(yg::launch_keyswitch(k, b->stream), "keyswitch launch");
    off = 0;
    for (const Part& part : take) {
        ck(cudaMemcpyAsync(part.r->h_out + (size_t)part.offset * n1, b->d_out + (size_t)off * n1,
                           (size_t)part.count * n1 * 4, cudaMemcpyDeviceToHost, b->stream),
           "copy out");
        off += part.count;
    }
    b->parts = std::move(take);
    b->tenants = std::move(used);
    b->refills = refills;
    s->refills_inflight += refills;
    s->refills_peak = std::max(s->refills_peak, s->refills_inflight);
    s->refill_sample_sum += s->refills_inflight;
    s->refill_samples++;
    b->busy = true;
    b->finished.store(false);
    ck(cudaLaunchHostFunc(b->stream, batch_done_cb, b), "completion callback");
    s->batches_run++;
    return true;
}

void worker_loop(yg_server* s) {
    if (cudaSetDevice(s->ctx->device) != cudaSuccess) return;
    std::deque<Request*> pending;
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        while (!s->incoming.empty()) {
            pending.push_back(s->incoming.front());
            s->incoming.pop_front();
        }
        retire(s);
        if (s->stopping && pending.empty() && std::none_of(s->batches.begin(), s->batches.end(),
                                                           [](const auto& b) { return b->busy; }))
            break;
        Batch* free_b = nullptr;
        for (auto& b : s->batches)
            if (!b->busy) {
                free_b = b.get();
                break;
            }
        bool launched = false;
        if (free_b && !pending.empty()) {
            try {
                launched = launch_batch(s, pending, free_b);
            } catch (const std::exception& e) {
                s->worker_error = e.what();
                s->stopping = true;
                for (Request* r : pending) r->done.store(true);
                pending.clear();
                s->cv_done.notify_all();
                break;
            }
        }
        if (!launched) s->cv.wait_for(lk, std::chrono::microseconds(500));
    }
}

// The first tenant's key is lazy: the slots are re-made for lazy keys ([half rows | table
// block] + KSK, so the budget holds more of them), with the kernel's per-slot key table and
// the transform tables in server memory (the key object may be destroyed after it is added).
void use_lazy_slots(yg_server* s, const yg_key* key) {
    const yg_params& p = s->ctx->p;
    const size_t cp = yg::lazy_cprime_bytes(p), tab_words = yg::lazy_tab_words(p, key->lazy_ls);
    const size_t bsk = cp + tab_words * 8;
    const int nslots = (int)(s->cfg.key_budget_bytes / (bsk + s->ksk_bytes));
    if (nslots < 1) throw std::invalid_argument("key budget smaller than one tenant's keys");
    for (auto* b : s->slot_bsk) cudaFree(b);
    for (auto* k : s->slot_ksk) cudaFree(k);
    s->slot_bsk.clear();
    s->slot_ksk.clear();
    s->slot_owner.clear();
    s->lazy = true;
    s->lazy_ls = key->lazy_ls;
    s->lazy_cprime_bytes = cp;
    s->bsk_bytes = bsk;
    s->nslots = nslots;
    std::vector<yg::LazyKeyRef> refs;
    for (int i = 0; i < nslots; i++) {
        uint32_t* b = nullptr;
        int32_t* k = nullptr;
        ck(cudaMalloc(&b, bsk), "key slot");
        s->slot_bsk.push_back(b);
        ck(cudaMalloc(&k, s->ksk_bytes), "key slot");
        s->slot_ksk.push_back(k);
        s->slot_owner.push_back(-1);
        const unsigned char* base = reinterpret_cast<const unsigned char*>(b);
        refs.push_back(yg::lazy_key_ref(p, base, reinterpret_cast<const uint64_t*>(base + cp), key->lazy_ls));
    }
    ck(cudaMalloc(&s->d_lazy_slot_table, refs.size() * sizeof(yg::LazyKeyRef)), "lazy slot table");
    ck(cudaMemcpy(s->d_lazy_slot_table, refs.data(), refs.size() * sizeof(yg::LazyKeyRef), cudaMemcpyHostToDevice),
       "lazy slot table");
    // the transforms' tables ([wi | wip | wf | wfp], N words each) are the same for every key
    ck(cudaMalloc(&s->d_lazy_tables, 4 * (size_t)p.N * 8), "lazy tables");
    ck(cudaMemcpy(s->d_lazy_tables, key->d_lazy_tab, 4 * (size_t)p.N * 8, cudaMemcpyDeviceToDevice), "lazy tables");
    s->lazy_tmpl = yg::lazy_launch_args(s->ctx, key);
    s->lazy_tmpl.cprime = nullptr;
    s->lazy_tmpl.s2 = s->lazy_tmpl.s2p = nullptr;
    s->lazy_tmpl.wi = s->d_lazy_tables;
    s->lazy_tmpl.wip = s->d_lazy_tables + p.N;
    s->lazy_tmpl.wf = s->d_lazy_tables + 2 * (size_t)p.N;
    s->lazy_tmpl.wfp = s->d_lazy_tables + 3 * (size_t)p.N;
}

}  // namespace

extern "C" {

int yg_server_create(yg_ctx* ctx, const yg_server_config* cfg, yg_server** out) {
    if (!ctx || !cfg || !out || cfg->max_batch < 1 || cfg->max_inflight < 1 || cfg->max_inflight > 8)
        return set_err(YG_ERR_INVALID, "yg_server_create: bad arguments");
    *out = nullptr;
    return guarded([&] {
        yg::DeviceGuard g(ctx->device);
        auto s = std::make_unique<yg_server>();
        s->ctx = ctx;
        s->cfg = *cfg;
        const yg_params& p = ctx->p;
        s->bsk_bytes = yg::key_words(p.n, p.l_approx, p.N) * 4;
        s->ksk_bytes = (size_t)p.k * p.N * p.ks_level * (p.n + 1) * 4;
        // GINX slots; a budget too small for them may still hold lazy keys (the first
        // tenant's family decides, use_lazy_slots)
        s->nslots = (int)(cfg->key_budget_bytes / (s->bsk_bytes + s->ksk_bytes));
        if (s->nslots < 1) s->nslots = 0;
        if (cfg->max_tenants < 1) throw std::invalid_argument("max_tenants must be positive");
        // small batches in the latency layout where the parameters have it
        if (cfg->latency_batch_max >= 0 && ctx->latency_max > 0)
            s->latency_max = cfg->latency_batch_max > 0 ? cfg->latency_batch_max : ctx->latency_max;
        auto fail_clean = [&]() {
            for (auto* b : s->slot_bsk) cudaFree(b);
            for (auto* k : s->slot_ksk) cudaFree(k);
            cudaFree(s->d_slot_table);
            cudaFree(s->d_lut_table);
            for (auto& b : s->batches) free_batch(b.get());
            if (s->copy) cudaStreamDestroy(s->copy);
        };
        try {
            for (int i = 0; i < s->nslots; i++) {
                uint32_t* b = nullptr;
                int32_t* k = nullptr;
                ck(cudaMalloc(&b, s->bsk_bytes), "key slot");
                s->slot_bsk.push_back(b);
                ck(cudaMalloc(&k, s->ksk_bytes), "key slot");
                s->slot_ksk.push_back(k);
                s->slot_owner.push_back(-1);
            }
            std::vector<const uint4*> table;
            for (uint32_t* b : s->slot_bsk) table.push_back(reinterpret_cast<const uint4*>(b));
            ck(cudaMalloc(&s->d_slot_table, std::max<size_t>(1, table.size()) * sizeof(void*)), "slot table");
            ck(cudaMemcpy(s->d_slot_table, table.data(), table.size() * sizeof(void*), cudaMemcpyHostToDevice),
               "slot table");
            ck(cudaMalloc(&s->d_lut_table, (size_t)cfg->max_tenants * sizeof(void*)), "LUT table");
            ck(cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking), "stream");
            const int n1 = p.n + 1, big = p.k * p.N + 1, mb = cfg->max_batch;
            for (int i = 0; i < cfg->max_inflight; i++) {
                auto b = std::make_unique<Batch>();
                b->server = s.get();
                ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
                ck(cudaMalloc(&b->d_in, (size_t)mb * n1 * 4), "batch buffer");
                ck(cudaMalloc(&b->d_out, (size_t)mb * n1 * 4), "batch buffer");
                ck(cudaMalloc(&b->d_big, (size_t)mb * big * 4), "batch buffer");
                ck(cudaMalloc(&b->d_key_of, (size_t)mb * 4), "batch buffer");
                ck(cudaMalloc(&b->d_lut_of, (size_t)mb * 4), "batch buffer");
                ck(cudaMalloc(&b->d_tiles, (size_t)mb * sizeof(yg::KsTile)), "batch buffer");
                ck(cudaMallocHost(&b->h_key_of, (size_t)mb * 4), "batch staging");
                ck(cudaMallocHost(&b->h_lut_of, (size_t)mb * 4), "batch staging");
                ck(cudaMallocHost(&b->h_tiles, (size_t)mb * sizeof(yg::KsTile)), "batch staging");
                s->batches.push_back(std::move(b));
            }
        } catch (...) {
            fail_clean();
            throw;
        }
        *out = s.release();
        return YG_OK;
    });
}

int yg_server_add_tenant(yg_server* s, int tenant, const yg_key* key, const int64_t* h_lut) {
    if (!s || !key || !h_lut || tenant < 0) return set_err(YG_ERR_INVALID, "yg_server_add_tenant: bad arguments");
    if (int rc = yg::check_key(s->ctx, key, true, true, true)) return rc;
    if (key->grouped()) return set_err(YG_ERR_INVALID, "yg_server_add_tenant: group keys run through yg_pbs");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return set_err(YG_ERR_STATE, "tenants must be added before yg_server_start");
    if (s->tenants.count(tenant)) return set_err(YG_ERR_INVALID, "tenant already registered");
    if ((int)s->by_index.size() >= s->cfg.max_tenants) return set_err(YG_ERR_INVALID, "too many tenants");
    if (s->family_set && (key->lazy() != s->lazy || key->lazy_ls != s->lazy_ls))
        return set_err(YG_ERR_INVALID, "yg_server_add_tenant: a server serves keys of one family (GINX or lazy)");
    return guarded([&] {
        yg::DeviceGuard g(s->ctx->device);
        if (!s->family_set && key->lazy()) use_lazy_slots(s, key);
        if (s->nslots < 1) throw std::invalid_argument("key budget smaller than one tenant's keys");
        s->family_set = true;
        auto t = std::make_unique<Tenant>();
        t->id = tenant;
        t->index = (int)s->by_index.size();
        try {
            ck(cudaMallocHost(&t->h_bsk, s->bsk_bytes), "pinned key image");
            ck(cudaMallocHost(&t->h_ksk, s->ksk_bytes), "pinned key image");
            if (s->lazy) {  // [half rows | table block], the slot's layout
                unsigned char* img = reinterpret_cast<unsigned char*>(t->h_bsk);
                ck(cudaMemcpy(img, key->d_lazy_cprime, s->lazy_cprime_bytes, cudaMemcpyDeviceToHost), "key image");
                ck(cudaMemcpy(img + s->lazy_cprime_bytes, key->d_lazy_tab, s->bsk_bytes - s->lazy_cprime_bytes,
                              cudaMemcpyDeviceToHost),
                   "key image");
            } else {
                ck(cudaMemcpy(t->h_bsk, key->d_bsk, s->bsk_bytes, cudaMemcpyDeviceToHost), "key image");
            }
            ck(cudaMemcpy(t->h_ksk, key->d_ksk, s->ksk_bytes, cudaMemcpyDeviceToHost), "key image");
            ck(cudaMalloc(&t->d_lut, (size_t)s->ctx->p.N * 8), "LUT");
            ck(cudaMemcpy(t->d_lut, h_lut, (size_t)s->ctx->p.N * 8, cudaMemcpyHostToDevice), "LUT");
            ck(cudaMemcpy(s->d_lut_table + t->index, &t->d_lut, sizeof(void*), cudaMemcpyHostToDevice), "LUT table");
            ck(cudaEventCreateWithFlags(&t->ready, cudaEventDisableTiming), "event");
        } catch (...) {
            cudaFreeHost(t->h_bsk);
            cudaFreeHost(t->h_ksk);
            cudaFree(t->d_lut);
            throw;
        }
        s->by_index.push_back(t.get());
        s->tenants[tenant] = std::move(t);
        return YG_OK;
    });
}

int yg_server_start(yg_server* s) {
    if (!s) return set_err(YG_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return YG_OK;
    s->running = true;
    s->stopping = false;
    s->busy_since = now_s();
    s->worker = std::thread(worker_loop, s);
    return YG_OK;
}

int64_t yg_server_submit(yg_server* s, int tenant, const int32_t* h_in, int32_t* h_out, int count) {
    if (!s || !h_in || !h_out || count < 1) return set_err(YG_ERR_INVALID, "yg_server_submit: bad arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->running || s->stopping) return set_err(YG_ERR_STATE, "server not running");
    if (count > s->cfg.max_batch) return set_err(YG_ERR_INVALID, "request larger than max_batch");
    if (!s->tenants.count(tenant)) return set_err(YG_ERR_INVALID, "unknown tenant");
    auto r = std::make_unique<Request>();
    r->id = s->next_id++;
    r->tenant = tenant;
    r->count = count;
    r->h_in = h_in;
    r->h_out = h_out;
    r->t_submit = now_s();
    Request* raw = r.get();
    s->requests[raw->id] = std::move(r);
    s->incoming.push_back(raw);
    s->waiting_peak = std::max(s->waiting_peak, ++s->waiting);
    s->cv.notify_all();
    return raw->id;
}

int yg_server_wait(yg_server* s, int64_t request, int timeout_ms, yg_request_times* times) {
    if (!s) return set_err(YG_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(request);
    if (it == s->requests.end()) return set_err(YG_ERR_INVALID, "unknown request");
    Request* r = it->second.get();
    const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 1 << 30 : timeout_ms),
                                        [&] { return r->done.load(); });
    if (!s->worker_error.empty()) return set_err(YG_ERR_CUDA, "server worker failed: " + s->worker_error);
    if (!ok) return set_err(YG_ERR_STATE, "timeout");
    if (times) {
        times->t_submit = r->t_submit;
        times->t_start = r->t_start;
        times->t_done = r->t_done;
    }
    s->requests.erase(it);
    return YG_OK;
}

int yg_server_stats(yg_server* s, yg_server_counters* out) {
    if (!s || !out) return set_err(YG_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    out->key_hits = s->hits;
    out->key_misses = s->misses;
    out->refill_bytes = s->refill_bytes;
    out->batches = s->batches_run;
    out->requests_done = s->requests_done;
    out->ciphertexts_done = s->ciphertexts_done;
    out->key_slots = s->nslots;
    out->latency_batches = s->latency_batches_run;
    return YG_OK;
}

void yg_server_destroy(yg_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    yg::DeviceGuard g(s->ctx->device);
    cudaStreamSynchronize(s->copy);
    for (auto& b : s->batches) free_batch(b.get());
    for (auto& kv : s->tenants) {
        Tenant* t = kv.second.get();
        cudaFreeHost(t->h_bsk);
        cudaFreeHost(t->h_ksk);
        cudaFree(t->d_lut);
        cudaEventDestroy(t->ready);
    }
    for (auto* b : s->slot_bsk) cudaFree(b);
    for (auto* k : s->slot_ksk) cudaFree(k);
    cudaFree(s->d_slot_table);
    cudaFree(s->d_lut_table);
    cudaFree(s->d_lazy_slot_table);
    cudaFree(s->d_lazy_tables);
    cudaStreamDestroy(s->copy);
    delete s;
}

}  // extern "C"

// ---------------------------------------------------------------------------- trace replay

namespace {

// Zipf(s) over ranks 0..n-1 by inverse CDF (ZipfDistribution, yatfhe/include/yautil/zipf.h:47-87):
// harmonic normalisation, cumulative table with the last entry set to 1, lower_bound of a
// uniform draw, ranks clamped to n-1.
struct Zipf {
    std::vector<double> cdf;
    std::mt19937_64 gen;
    std::uniform_real_distribution<double> uni{0.0, 1.0};
    Zipf(double s, int n, uint64_t seed) : cdf(n), gen(seed) {
        double h = 0;
        for (int k = 1; k <= n; k++) h += 1.0 / std::pow(k, s);
        double c = 0;
        for (int r = 1; r <= n; r++) {
            c += 1.0 / (std::pow(r, s) * h);
            cdf[r - 1] = c;
        }
        cdf[n - 1] = 1.0;
    }
    int next() {
        const double u = uni(gen);
        int r = (int)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        return std::min(r, (int)cdf.size() - 1);
    }
};

yg_latency summarize(std::vector<double> v) {
    yg_latency o{};
    if (v.empty()) return o;
    std::sort(v.begin(), v.end());
    double sum = 0;
    for (double x : v) sum += x;
    auto pct = [&](double p) {
        long i = (long)std::ceil(p / 100.0 * v.size()) - 1;
        return v[std::min<long>(std::max<long>(i, 0), (long)v.size() - 1)];
    };
    o.mean_ms = sum / v.size();
    o.p50_ms = pct(50);
    o.p90_ms = pct(90);
    o.p99_ms = pct(99);
    o.p999_ms = pct(99.9);
    o.max_ms = v.back();
    return o;
}

}  // namespace

extern "C" int yg_server_run_trace(yg_server* s, const yg_trace_config* cfg, yg_trace_result* out) {
    if (!s || !cfg || !out || cfg->requests < 1 || cfg->warmup < 0 || cfg->rate <= 0 || cfg->tenants < 1 ||
        cfg->max_count < 1 || cfg->max_count > s->cfg.max_batch || !cfg->h_pool)
        return set_err(YG_ERR_INVALID, "yg_server_run_trace: bad arguments");
    for (int t = 0; t < cfg->tenants; t++)
        if (!s->tenants.count(t)) return set_err(YG_ERR_INVALID, "trace tenant not registered");
    return guarded([&] {
        yg::DeviceGuard g(s->ctx->device);
        const int n1 = s->ctx->p.n + 1;
        const size_t req_words = (size_t)cfg->max_count * n1;
        const int total = cfg->warmup + cfg->requests;
        // pinned output ring, one slot per request in flight
        const int ring = 512;
        int32_t* h_out = nullptr;
        ck(cudaMallocHost(&h_out, (size_t)ring * req_words * 4), "output ring");
        std::unique_ptr<int32_t, decltype(&cudaFreeHost)> ring_guard(h_out, &cudaFreeHost);
        std::mutex fm;
        std::condition_variable fcv;
        std::deque<int> free_slots;
        for (int i = 0; i < ring; i++) free_slots.push_back(i);

        struct Issued {
            int64_t id;
            Request* req;
            int slot, tenant, count;
            bool measured;
        };
        std::mutex qm;
        std::condition_variable qcv;
        std::deque<Issued> issued;
        bool producer_done = false;
        std::atomic<int> shed{0};
        std::atomic<bool> aborted{false};  // the consumer hit an error: the producer stops
        std::atomic<int> in_system{0};     // submitted and not yet reaped

        if (int rc = yg_server_start(s)) return rc;
        yg_server_counters before{};
        yg_server_counters after{};
        std::vector<double> soj, que, svc;
        std::map<int, std::pair<double, long>> per_tenant;  // sum of sojourn (ms), requests
        int mismatched = 0, served = 0;
        double t_first = 0, t_last = 0;
        int64_t measured_cts = 0;

        std::thread producer([&] {
            std::mt19937_64 arrivals(cfg->seed ^ 0x9e3779b97f4a7c15ULL);
            std::exponential_distribution<double> gap(1.0);
            std::mt19937_64 sizes(cfg->seed + 1);
            std::uniform_real_distribution<double> lsz(0.0, std::log((double)cfg->max_count + 1.0));
            Zipf zipf(cfg->zipf_s, cfg->tenants, cfg->zipf_seed);
            const auto t0 = Clock::now();
            double offset = 0;
            for (int i = 0; i < total; i++) {
                offset += gap(arrivals) / cfg->rate;
                std::this_thread::sleep_until(t0 + std::chrono::duration_cast<Clock::duration>(
                                                       std::chrono::duration<double>(offset)));
                const int tenant = zipf.next();
                const int count = std::min(cfg->max_count, std::max(1, (int)std::floor(std::exp(lsz(sizes)))));
                if (cfg->queue_max > 0 && in_system.load() > cfg->queue_max) {
                    shed++;
                    continue;
                }
                int slot;
                {
                    std::unique_lock<std::mutex> lk(fm);
                    fcv.wait(lk, [&] { return !free_slots.empty() || aborted.load(); });
                    if (aborted.load()) break;
                    slot = free_slots.front();
                    free_slots.pop_front();
                }
                const int32_t* in = cfg->h_pool + (size_t)tenant * req_words;
                if (i == cfg->warmup) {  // counters of the measured window
                    yg_server_stats(s, &before);
                    std::lock_guard<std::mutex> lk(s->mu);
                    s->waiting_peak = s->waiting;
                    s->refills_peak = s->refills_inflight;
                    s->refill_samples = s->refill_sample_sum = 0;
                }
                const int64_t id = yg_server_submit(s, tenant, in, h_out + (size_t)slot * req_words, count);
                if (id <= 0) break;
                in_system++;
                Request* req;
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    req = s->requests[id].get();
                }
                std::lock_guard<std::mutex> lk(qm);
                issued.push_back(Issued{id, req, slot, tenant, count, i >= cfg->warmup});
                qcv.notify_all();
            }
            std::lock_guard<std::mutex> lk(qm);
            producer_done = true;
            qcv.notify_all();
        });

        // Completions are reaped in whatever order they happen, and each frees its output
        // slot at once: a request that waits long (a cold tenant) must not hold back the
        // slots of the requests behind it, or the producer would stop offering load.
        int err = YG_OK;
        std::vector<Issued> outstanding;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(qm);
                qcv.wait_for(lk, std::chrono::milliseconds(1), [&] { return !issued.empty() || producer_done; });
                while (!issued.empty()) {
                    outstanding.push_back(issued.front());
                    issued.pop_front();
                }
                if (outstanding.empty()) {
                    if (producer_done) break;
                    continue;
                }
            }
            bool failed = false;
            {
                std::unique_lock<std::mutex> lk(s->mu);
                s->cv_done.wait_for(lk, std::chrono::milliseconds(1), [&] {
                    failed = !s->worker_error.empty();
                    if (failed) return true;
                    for (const Issued& it : outstanding)
                        if (it.req->done.load()) return true;
                    return false;
                });
            }
            for (size_t k = 0; k < outstanding.size();) {
                const Issued it = outstanding[k];
                if (!failed && !it.req->done.load()) {
                    k++;
                    continue;
                }
                outstanding[k] = outstanding.back();
                outstanding.pop_back();
                in_system--;
                yg_request_times tm{};
                const int rc = yg_server_wait(s, it.id, 600000, &tm);
                if (rc != YG_OK) {
                    err = rc;
                    break;
                }
                const int32_t* o = h_out + (size_t)it.slot * req_words;
                if (cfg->h_expect &&
                    std::memcmp(o, cfg->h_expect + (size_t)it.tenant * req_words, (size_t)it.count * n1 * 4) != 0)
                    mismatched++;
                if (it.measured) {
                    t_first = served == 0 ? tm.t_submit : std::min(t_first, tm.t_submit);
                    served++;
                    measured_cts += it.count;
                    t_last = std::max(t_last, tm.t_done);
                    soj.push_back(1e3 * (tm.t_done - tm.t_submit));
                    auto& pt = per_tenant[it.tenant];
                    pt.first += soj.back();
                    pt.second++;
                    que.push_back(1e3 * (tm.t_start - tm.t_submit));
                    svc.push_back(1e3 * (tm.t_done - tm.t_start));
                }
                std::lock_guard<std::mutex> lk(fm);
                free_slots.push_back(it.slot);
                fcv.notify_all();
            }
            if (err != YG_OK) {
                {
                    std::lock_guard<std::mutex> lk(fm);
                    aborted.store(true);
                }
                fcv.notify_all();
                break;
            }
        }
        producer.join();
        if (err != YG_OK) return err;
        yg_server_stats(s, &after);
        std::memset(out, 0, sizeof(*out));
        out->served = served;
        out->shed = shed.load();
        out->mismatched_requests = mismatched;
        out->seconds = t_last - t_first;
        out->requests_per_s = out->seconds > 0 ? served / out->seconds : 0;
        out->ciphertexts_per_s = out->seconds > 0 ? measured_cts / out->seconds : 0;
        out->offered_rate = cfg->rate;
        out->sojourn = summarize(soj);
        out->queue = summarize(que);
        out->service = summarize(svc);
        out->key_hits = after.key_hits - before.key_hits;
        out->key_misses = after.key_misses - before.key_misses;
        out->refill_bytes = after.refill_bytes - before.refill_bytes;
        out->batches = after.batches - before.batches;
        out->latency_batches = after.latency_batches - before.latency_batches;
        const double lookups = (double)(out->key_hits + out->key_misses);
        out->hit_rate = lookups > 0 ? out->key_hits / lookups : 0;
        // the reference's SLO and fairness figures (blindrotate_serving.cpp:256-284, 324-336)
        out->slo_ms = cfg->slo_ms > 0 ? cfg->slo_ms : 100.0;
        auto violation = [&](double budget) {
            size_t v = 0;
            for (double x : soj) v += x > budget;
            return soj.empty() ? 0.0 : (double)v / soj.size();
        };
        out->slo_violation_rate = violation(out->slo_ms);
        out->slo_violation_rate_100 = violation(100.0);
        out->slo_violation_rate_300 = violation(300.0);
        out->slo_violation_rate_500 = violation(500.0);
        out->tenant_fairness_jain = 1.0;
        if (per_tenant.size() > 1) {
            double sum = 0, sum_sq = 0;
            for (const auto& e : per_tenant) {
                const double m = e.second.first / e.second.second;
                sum += m;
                sum_sq += m * m;
            }
            out->tenant_fairness_jain = sum * sum / (per_tenant.size() * sum_sq);
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            out->peak_queue_depth = s->waiting_peak;
            out->load_concurrency_peak = s->refills_peak;
            out->load_concurrency_mean =
                s->refill_samples ? (double)s->refill_sample_sum / s->refill_samples : 0.0;
        }
        return YG_OK;
    });
}
