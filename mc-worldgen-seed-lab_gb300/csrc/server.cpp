/* server.cpp -- the served form: continuous batching of biome-map requests (mcgen_gb300_server_*).
 *
 * Callers submit requests (world, seed, quart region) from any thread at any time and get a ticket.  A
 * worker thread admits every pending request into the next batch as soon as one of the server's streams
 * is free (up to `max_inflight` batches run at once, so a batch that forms while another is on the GPU
 * starts right away and the two overlap on the device), makes sure each request's seed lattices are
 * resident in the device noise-state cache, enqueues the setup launches for the cache misses and one
 * persistent k_batch launch, and copies the ids back.  When a batch's event completes the worker hands
 * every request its ids and wakes its waiters.
 *
 * Noise-state cache: per dimension a pool of fixed-size slots (46 lattices of 352 B for the Overworld, 8 for
 * the Nether, 1 for the End) carved from one HBM budget, keyed by (world identity, seed) -- the world's
 * process-unique id, never its address, which the heap may give to a later world -- and evicted least
 * recently used among slots that no in-flight batch references.
 *
 * Failures: a batch that fails before its work is queued (an allocation, a copy or a launch) takes back the
 * cache entries it had created, so no later request can hit lattices that were never built, and fails its
 * own requests; an allocation failure leaves the server usable, any other error stops it: every pending
 * and later request then fails with that error.  A pending request holds its world, so mcgen_world_free
 * during serving defers the free until the request completes.
 */
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/mcgen_gb300.h"
#include "abi_internal.h"
#include "batch.h"
#include "launch.h"

namespace {

using Clock = std::chrono::steady_clock;

using Key = std::pair<uint64_t, int64_t>; /* (world uid, seed) */

struct Pool { /* one dimension's slots */
    int lattices_per_slot = 0;
    int nslots = 0;
    MgLattice *base = nullptr;
    std::vector<int> free_slots;
    std::list<Key> lru; /* front = most recent */
    /* builder: the batch slot whose setup launch is still filling this entry, -1 once it is complete */
    struct Entry { int slot; int refs; int builder; std::list<Key>::iterator it; };
    std::map<Key, Entry> map;
};

struct Ticket {
    McGb300Request req;
    uint8_t *out;
    Clock::time_point t_submit, t_done;
    int state = 0; /* 0 pending, 1 running, 2 done, 3 failed */
    int err = 0;
};

struct Batch {
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t setup_done = nullptr; /* after this batch's setup launches */
    bool busy = false;
    std::vector<long long> tickets;
    std::vector<std::pair<int, Key>> held; /* (dim, key) references */
    /* device and pinned staging, grown as needed */
    MgBatchReq *d_reqs = nullptr; size_t cap_reqs = 0;
    MgSetupEntry *d_ent = nullptr; size_t cap_ent = 0;
    int *d_first = nullptr; size_t cap_first = 0;
    MgWorldDesc *d_worlds = nullptr; size_t cap_worlds = 0;
    const MgTreeNode **d_trees = nullptr;
    uint8_t *d_out = nullptr; size_t cap_out = 0;
    uint8_t *h_out = nullptr; size_t cap_hout = 0;
    unsigned long long *d_counter = nullptr; /* tiles taken, cells recorded for the exact pass */
    MgPending *d_pend = nullptr; size_t cap_pend = 0;
    std::vector<long long> out_off;
};

}  // namespace

struct McGb300Server {
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    int max_batch = 4096;
    Pool pool[3];
    std::vector<Batch> batches;
    std::deque<long long> pending;
    std::unordered_map<long long, Ticket> tickets;
    long long next_ticket = 1;
    McGb300ServerStats stats;
    int fatal = 0;
    int fail_next = 0; /* testing aid: the next batch's allocation step fails with this code */
};

namespace {

/* tile shape of the served batches: 8 x 16 cells at 6 resident CTAs per SM, the shape the autotuner picks
 * for the uneven mixed batch */
const int kServeShape = 2;

int crc(cudaError_t e) { return e == cudaSuccess ? 0 : e == cudaErrorMemoryAllocation ? MCGEN_E_NOMEM : MCGEN_E_INTERNAL; }

template <typename T>
cudaError_t grow_dev(T **p, size_t *cap, size_t n) {
    if (n <= *cap) return cudaSuccess;
    size_t c = n + n / 2 + 16;
    cudaFree((void *)*p);
    *p = nullptr;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * c);
    *cap = e ? 0 : c;
    return e;
}

/* Reserve a cache slot for key in pool P (caller holds the server lock); -1 if every slot is in use.
 * *builder: the batch still building a hit entry (-1 when complete); a miss is built by batch `me`. */
int cache_acquire(McGb300Server *s, Pool &P, const Key &key, int me, bool *miss, int *builder) {
    auto it = P.map.find(key);
    if (it != P.map.end()) {
        it->second.refs++;
        P.lru.erase(it->second.it);
        P.lru.push_front(key);
        it->second.it = P.lru.begin();
        *miss = false;
        *builder = it->second.builder;
        s->stats.cache_hits++;
        return it->second.slot;
    }
    int slot = -1;
    if (!P.free_slots.empty()) {
        slot = P.free_slots.back();
        P.free_slots.pop_back();
    } else {
        for (auto r = P.lru.rbegin(); r != P.lru.rend(); ++r) { /* least recently used, unreferenced */
            auto e = P.map.find(*r);
            if (e->second.refs == 0) {
                slot = e->second.slot;
                P.lru.erase(std::next(r).base());
                P.map.erase(e);
                s->stats.cache_evictions++;
                break;
            }
        }
        if (slot < 0) return -1;
    }
    P.lru.push_front(key);
    P.map[key] = Pool::Entry{slot, 1, me, P.lru.begin()};
    *miss = true;
    *builder = -1;
    s->stats.cache_misses++;
    return slot;
}
void cache_release(Pool &P, const Key &key, int me) {
    auto it = P.map.find(key);
    if (it == P.map.end()) return;
    if (it->second.refs > 0) it->second.refs--;
    if (it->second.builder == me) it->second.builder = -1; /* its batch has completed */
}
/* A batch that failed before its work was queued: entries it created were never built, so they leave the
 * cache (their slots return to the free list); other entries just lose this batch's references.  No other
 * batch can reference an entry this batch created: batches form one at a time under the server lock. */
void cache_rollback(Pool &P, const Key &key, int me) {
    auto it = P.map.find(key);
    if (it == P.map.end()) return;
    if (it->second.refs > 0) it->second.refs--;
    if (it->second.builder == me) {
        P.free_slots.push_back(it->second.slot);
        P.lru.erase(it->second.it);
        P.map.erase(it);
    }
}

/* A request has completed or failed: record it and let go of its world (caller holds the server lock and
 * the ABI lock). */
void ticket_done(Ticket &T, int err, Clock::time_point now) {
    T.state = err ? 3 : 2;
    T.err = err;
    T.t_done = now;
    mg::abi_world_release(const_cast<McWorld *>(T.req.world));
}

/* Form and launch one batch from pending requests on batch slot b (server lock held). */
int launch_batch(McGb300Server *s, Batch &b) {
    const int me = (int)(&b - s->batches.data());
    std::vector<int> wait_on;
    std::vector<const McWorld *> worlds;
    std::map<const McWorld *, int> widx;
    std::vector<MgBatchReq> reqs;
    std::vector<MgSetupEntry> ent[3];
    std::vector<int> first;
    long long tiles = 0, out = 0, ow = 0;
    b.tickets.clear();
    b.held.clear();
    b.out_off.clear();
    while (!s->pending.empty() && (int)b.tickets.size() < s->max_batch) {
        const long long id = s->pending.front();
        Ticket &T = s->tickets[id];
        const McWorld *w = T.req.world;
        const int dim = w->desc.dim;
        const Key key = std::make_pair(w->uid, (int64_t)T.req.seed);
        Pool &P = s->pool[dim];
        if (w->desc.ntables > P.lattices_per_slot) { /* cannot happen with the shipped tables */
            s->pending.pop_front();
            ticket_done(T, MCGEN_E_DATA, Clock::now());
            s->cv_done.notify_all();
            continue;
        }
        bool miss = false;
        int builder = -1;
        /* the same key twice in one batch is one reference per request */
        const int slot = cache_acquire(s, P, key, me, &miss, &builder);
        if (slot < 0) break; /* cache full of in-flight states: wait for a batch to finish */
        if (builder >= 0 && builder != me) wait_on.push_back(builder);
        s->pending.pop_front();
        b.held.push_back(std::make_pair(dim, key));
        if (!widx.count(w)) { widx[w] = (int)worlds.size(); worlds.push_back(w); }
        const int lat = (int)((P.base - s->pool[0].base) + (long long)slot * P.lattices_per_slot);
        if (miss) {
            MgSetupEntry e;
            e.seed = T.req.seed;
            e.world = widx[w];
            e.slot = lat;
            if (dim == MG_OVERWORLD) { first.push_back((int)ow); ow += w->desc.ntables; }
            ent[dim].push_back(e);
        }
        MgBatchReq r;
        r.world = widx[w];
        r.state = lat;
        r.qx0 = T.req.qx0; r.qz0 = T.req.qz0; r.nx = T.req.nx; r.nz = T.req.nz; r.qy = T.req.qy;
        r.tie = MG_TIE_ENGINE;
        r.tile0 = 0;
        r.out_off = out;
        b.out_off.push_back(out);
        out += (long long)r.nx * r.nz;
        reqs.push_back(r);
        b.tickets.push_back(id);
        T.state = 1;
    }
    if (b.tickets.empty()) return 0;
    /* processing order grouped by code path, heaviest first (as in a plan), then the tile numbering */
    std::stable_sort(reqs.begin(), reqs.end(), [&](const MgBatchReq &x, const MgBatchReq &y) {
        const MgWorldDesc &a = worlds[(size_t)x.world]->desc, &c = worlds[(size_t)y.world]->desc;
        const int wa = a.dim * 2 + (a.fmode ? 1 : 0), wc = c.dim * 2 + (c.fmode ? 1 : 0);
        return wa != wc ? wa < wc : x.world < y.world;
    });
    for (auto &r : reqs) {
        r.tile0 = tiles;
        tiles += mg::batch_tiles(worlds[(size_t)r.world]->desc.dim, r.qx0, r.qz0, r.nx, r.nz, kServeShape);
    }
    cudaError_t e = cudaSuccess;
    std::vector<MgWorldDesc> wd;
    std::vector<const MgTreeNode *> tp;
    for (auto *w : worlds) { wd.push_back(w->desc); tp.push_back(w->d_tree); }
    size_t ntrees_cap = b.cap_worlds;
    if (!e) e = grow_dev(&b.d_worlds, &b.cap_worlds, wd.size());
    if (!e && b.cap_worlds != ntrees_cap) {
        cudaFree((void *)b.d_trees);
        b.d_trees = nullptr;
        e = cudaMalloc((void **)&b.d_trees, sizeof(void *) * b.cap_worlds);
    }
    size_t ent_n = ent[0].size() + ent[1].size() + ent[2].size();
    if (!e) e = grow_dev(&b.d_reqs, &b.cap_reqs, reqs.size());
    if (!e) e = grow_dev(&b.d_ent, &b.cap_ent, ent_n ? ent_n : 1);
    if (!e) e = grow_dev(&b.d_first, &b.cap_first, first.size() ? first.size() : 1);
    if (!e) e = grow_dev(&b.d_out, &b.cap_out, (size_t)out);
    if (!e && (size_t)out > b.cap_hout) {
        cudaFreeHost(b.h_out);
        b.h_out = nullptr;
        size_t c = (size_t)out + (size_t)out / 2;
        e = cudaMallocHost((void **)&b.h_out, c);
        b.cap_hout = e ? 0 : c;
    }
    if (!e && !b.d_counter) e = cudaMalloc(&b.d_counter, 2 * sizeof(unsigned long long));
    long long dcells = 0; /* double-branch Overworld cells: the ones the exact pass may take */
    for (const auto &r : reqs) {
        const MgWorldDesc &W = worlds[(size_t)r.world]->desc;
        if (W.dim == MG_OVERWORLD && !W.fmode) dcells += (long long)r.nx * r.nz;
    }
    const long long pend_cap = mg::batch_pending_cap(dcells);
    if (!e && pend_cap > 0) e = grow_dev(&b.d_pend, &b.cap_pend, (size_t)pend_cap);
    if (e) return crc(e);
    if (s->fail_next) { /* injected failure of this step (tests of the failure path) */
        const int f = s->fail_next;
        s->fail_next = 0;
        return f;
    }
    /* small host->device copies of this batch's descriptors (pageable sources: staged by the driver) */
    cudaStream_t st = b.st;
    e = cudaMemcpyAsync(b.d_worlds, wd.data(), sizeof(MgWorldDesc) * wd.size(), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync((void *)b.d_trees, tp.data(), sizeof(void *) * tp.size(), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(b.d_reqs, reqs.data(), sizeof(MgBatchReq) * reqs.size(), cudaMemcpyHostToDevice, st);
    size_t eo = 0;
    for (int d = 0; d < 3 && !e; d++) {
        if (ent[d].empty()) continue;
        e = cudaMemcpyAsync(b.d_ent + eo, ent[d].data(), sizeof(MgSetupEntry) * ent[d].size(), cudaMemcpyHostToDevice, st);
        eo += ent[d].size();
    }
    if (!e && !first.empty()) e = cudaMemcpyAsync(b.d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice, st);
    if (e) return crc(e);
    eo = 0;
    for (int d = 0; d < 3; d++) {
        if (ent[d].empty()) continue;
        int rc = mg::launch_setup_list(b.d_worlds, d, b.d_ent + eo, (int)ent[d].size(), b.d_first, ow, s->pool[0].base, st);
        if (rc) return MCGEN_E_INTERNAL;
        eo += ent[d].size();
    }
    if ((e = cudaEventRecord(b.setup_done, st))) return crc(e);
    /* hits on states another in-flight batch is still building: order after that batch's setup */
    for (int k : wait_on)
        if ((e = cudaStreamWaitEvent(st, s->batches[(size_t)k].setup_done, 0))) return crc(e);
    int rc = mg::launch_batch(b.d_worlds, b.d_trees, b.d_reqs, (int)reqs.size(), tiles, s->pool[0].base, b.d_counter,
                              pend_cap > 0 ? b.d_pend : nullptr, pend_cap, b.d_out, 0, kServeShape, st);
    if (rc) return MCGEN_E_INTERNAL;
    if ((e = cudaMemcpyAsync(b.h_out, b.d_out, (size_t)out, cudaMemcpyDeviceToHost, st))) return crc(e);
    if ((e = cudaEventRecord(b.done, st))) return crc(e);
    b.busy = true;
    s->stats.batches++;
    s->stats.requests_admitted += (long long)b.tickets.size();
    return 0;
}

/* Hand a finished batch's ids to its requests (server lock held).  launched: the batch's work was queued
 * (false: it failed while forming, and the cache entries it created are taken back). */
void finish_batch(McGb300Server *s, Batch &b, int err, bool launched) {
    const auto now = Clock::now();
    std::lock_guard<std::mutex> glk(mg::abi_lock());
    for (size_t i = 0; i < b.tickets.size(); i++) {
        auto it = s->tickets.find(b.tickets[i]);
        if (it == s->tickets.end()) continue;
        Ticket &T = it->second;
        if (!err && T.out) memcpy(T.out, b.h_out + b.out_off[i], (size_t)T.req.nx * (size_t)T.req.nz);
        ticket_done(T, err, now);
        if (!err) s->stats.samples_done += (long long)T.req.nx * T.req.nz;
    }
    const int me = (int)(&b - s->batches.data());
    for (auto &h : b.held) {
        if (launched && !err) cache_release(s->pool[h.first], h.second, me);
        else cache_rollback(s->pool[h.first], h.second, me);
    }
    b.tickets.clear();
    b.held.clear();
    b.busy = false;
    s->cv_done.notify_all();
}

/* After an error that stops the server: every pending request fails with it (server lock held). */
void fail_pending(McGb300Server *s) {
    const auto now = Clock::now();
    std::lock_guard<std::mutex> glk(mg::abi_lock());
    while (!s->pending.empty()) {
        auto it = s->tickets.find(s->pending.front());
        s->pending.pop_front();
        if (it != s->tickets.end()) ticket_done(it->second, s->fatal, now);
    }
    s->cv_done.notify_all();
}

void worker_loop(McGb300Server *s) {
    std::unique_lock<std::mutex> lk(s->m);
    for (;;) {
        bool progressed = false;
        /* completions */
        for (auto &b : s->batches) {
            if (!b.busy) continue;
            cudaError_t q = cudaEventQuery(b.done);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess && !s->fatal) s->fatal = MCGEN_E_INTERNAL; /* the device failed the batch */
            finish_batch(s, b, q == cudaSuccess ? 0 : MCGEN_E_INTERNAL, true);
            progressed = true;
        }
        if (s->fatal && !s->pending.empty()) {
            fail_pending(s);
            progressed = true;
        }
        /* admissions: every free stream takes the pending requests */
        for (auto &b : s->batches) {
            if (b.busy || s->pending.empty() || s->fatal) continue;
            int rc;
            {
                std::lock_guard<std::mutex> glk(mg::abi_lock());
                rc = launch_batch(s, b);
            }
            if (rc) { /* fail the requests of this batch loudly; its cache entries are taken back */
                finish_batch(s, b, rc, false);
                if (rc != MCGEN_E_NOMEM) {
                    s->fatal = rc;
                    fail_pending(s);
                }
                progressed = true;
            } else if (b.busy) {
                progressed = true;
            }
            /* not busy and no error: the cache is full of states that running batches use; wait for one */
        }
        if (s->stop && s->pending.empty()) {
            bool any = false;
            for (auto &b : s->batches) any |= b.busy;
            if (!any) return;
        }
        bool busy = false;
        for (auto &b : s->batches) busy |= b.busy;
        if (!progressed) {
            if (busy) { /* poll the running batches; new requests also wake us */
                s->cv_work.wait_for(lk, std::chrono::microseconds(50));
            } else {
                s->cv_work.wait(lk, [s] { return s->stop || !s->pending.empty(); });
            }
        }
    }
}

}  // namespace

extern "C" {

MCGEN_API int mcgen_gb300_server_new(long long hbm_budget_bytes, int max_inflight, int max_batch_requests,
                                     McGb300Server **out) {
    if (!out || hbm_budget_bytes < (long long)(64 * sizeof(MgLattice)) || max_inflight < 1 || max_inflight > 8)
        return MCGEN_E_ARG;
    *out = nullptr;
    std::lock_guard<std::mutex> glk(mg::abi_lock());
    if (!mg::abi_device_ready()) return MCGEN_E_UNSUPPORTED;
    McGb300Server *s = new McGb300Server();
    memset(&s->stats, 0, sizeof s->stats);
    s->max_batch = max_batch_requests > 0 ? max_batch_requests : 4096;
    /* budget split: Overworld 3/4, Nether 3/16, End 1/16 of the lattices */
    const long long lat_total = hbm_budget_bytes / (long long)sizeof(MgLattice);
    const int lps[3] = {48, 8, 1}; /* lattices per seed: Overworld 46, Nether 8, End 1 */
    const long long share[3] = {lat_total * 12 / 16, lat_total * 3 / 16, lat_total / 16};
    long long total = 0;
    for (int d = 0; d < 3; d++) {
        s->pool[d].lattices_per_slot = lps[d];
        s->pool[d].nslots = (int)std::max(1LL, std::min(share[d] / lps[d], (long long)INT32_MAX / 64));
        total += (long long)s->pool[d].nslots * lps[d];
    }
    if (total > INT32_MAX) { delete s; return MCGEN_E_ARG; }
    MgLattice *base = nullptr;
    cudaError_t e = cudaMalloc(&base, sizeof(MgLattice) * (size_t)total);
    if (e) { delete s; return crc(e); }
    long long at = 0;
    for (int d = 0; d < 3; d++) {
        s->pool[d].base = base + at;
        at += (long long)s->pool[d].nslots * lps[d];
        for (int i = s->pool[d].nslots - 1; i >= 0; i--) s->pool[d].free_slots.push_back(i);
    }
    s->stats.cache_slots[0] = s->pool[0].nslots;
    s->stats.cache_slots[1] = s->pool[1].nslots;
    s->stats.cache_slots[2] = s->pool[2].nslots;
    mg::batch_prepare(nullptr); /* kernel attributes and resident grids, before any launch */
    s->batches.resize((size_t)max_inflight);
    for (auto &b : s->batches) {
        if ((e = cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking)) ||
            (e = cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming)) ||
            (e = cudaEventCreateWithFlags(&b.setup_done, cudaEventDisableTiming))) {
            cudaFree(base);
            delete s;
            return crc(e);
        }
    }
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return MCGEN_OK;
}

MCGEN_API void mcgen_gb300_server_free(McGb300Server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->worker.join();
    std::lock_guard<std::mutex> glk(mg::abi_lock());
    for (auto &b : s->batches) {
        cudaStreamSynchronize(b.st);
        cudaStreamDestroy(b.st);
        cudaEventDestroy(b.done);
        cudaEventDestroy(b.setup_done);
        cudaFree(b.d_reqs);
        cudaFree(b.d_ent);
        cudaFree(b.d_first);
        cudaFree(b.d_worlds);
        cudaFree((void *)b.d_trees);
        cudaFree(b.d_out);
        cudaFreeHost(b.h_out);
        cudaFree(b.d_counter);
        cudaFree(b.d_pend);
    }
    cudaFree(s->pool[0].base);
    delete s;
}

MCGEN_API int mcgen_gb300_server_submit(McGb300Server *s, const McGb300Request *req, uint8_t *out, long long *ticket) {
    if (!s || !req || !req->world || !out || !ticket || req->nx <= 0 || req->nz <= 0 ||
        (long long)req->nx * req->nz > (1LL << 28))
        return MCGEN_E_ARG;
    {
        /* the world's tree must be on the device before the worker references it, and the world stays alive
         * until the request completes */
        std::lock_guard<std::mutex> glk(mg::abi_lock());
        int rc = mg::abi_world_device(const_cast<McWorld *>(req->world));
        if (rc) return rc;
        mg::abi_world_hold(const_cast<McWorld *>(req->world));
    }
    std::lock_guard<std::mutex> lk(s->m);
    if (s->fatal) {
        std::lock_guard<std::mutex> glk(mg::abi_lock());
        mg::abi_world_release(const_cast<McWorld *>(req->world));
        return s->fatal;
    }
    const long long id = s->next_ticket++;
    Ticket &T = s->tickets[id];
    T.req = *req;
    T.out = out;
    T.t_submit = Clock::now();
    s->pending.push_back(id);
    *ticket = id;
    s->stats.requests_submitted++;
    s->cv_work.notify_one();
    return MCGEN_OK;
}

MCGEN_API int mcgen_gb300_server_wait(McGb300Server *s, long long ticket, int timeout_ms, double *latency_ms) {
    if (!s) return MCGEN_E_ARG;
    std::unique_lock<std::mutex> lk(s->m);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return MCGEN_E_ARG;
    auto done = [&] { return it->second.state >= 2; };
    if (timeout_ms < 0) s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return MCGEN_E_CANCEL;
    const Ticket &T = it->second;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(T.t_done - T.t_submit).count();
    const int err = T.state == 3 ? (T.err ? T.err : MCGEN_E_INTERNAL) : MCGEN_OK;
    s->tickets.erase(it);
    return err;
}

/* Open-loop replay of an arrival schedule (a load generator for measuring the served form): a native thread
 * submits request i at t0 + arrival_s[i] (sleeping until shortly before, then spinning), the calling thread
 * waits for the tickets in order; latency_ms[i] runs from the scheduled arrival to the completion the server
 * records, so a submitter behind schedule adds to the latency instead of hiding it. */
MCGEN_API int mcgen_gb300_server_replay(McGb300Server *s, const McGb300Request *reqs, const double *arrival_s, int n,
                                        uint8_t *out, const long long *out_off, double *latency_ms, double *elapsed_s) {
    if (!s || n < 0 || (n > 0 && (!reqs || !arrival_s || !out || !out_off || !latency_ms))) return MCGEN_E_ARG;
    std::vector<long long> tk((size_t)n, -1);
    std::vector<Clock::time_point> sub((size_t)n);
    std::atomic<int> submitted{0};
    std::atomic<bool> done{false};
    std::atomic<int> sub_err{0};
    const auto t0 = Clock::now();
    auto due_of = [&](int i) {
        return t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
    };
    std::thread submitter([&] {
        for (int i = 0; i < n; i++) {
            const auto due = due_of(i);
            const auto early = due - std::chrono::microseconds(80);
            if (Clock::now() < early) std::this_thread::sleep_until(early);
            while (Clock::now() < due) {
            }
            sub[(size_t)i] = Clock::now();
            long long t = -1;
            const int rc = mcgen_gb300_server_submit(s, &reqs[i], out + out_off[i], &t);
            tk[(size_t)i] = rc ? -1 : t;
            submitted.store(i + 1, std::memory_order_release);
            if (rc) {
                sub_err = rc;
                break;
            }
        }
        done.store(true, std::memory_order_release);
    });
    int rc_all = 0;
    for (int i = 0; i < n; i++) {
        while (submitted.load(std::memory_order_acquire) <= i && !done.load(std::memory_order_acquire))
            std::this_thread::yield();
        if (submitted.load(std::memory_order_acquire) <= i || tk[(size_t)i] < 0) break; /* the submitter stopped */
        double ms = 0.0;
        const int rc = mcgen_gb300_server_wait(s, tk[(size_t)i], -1, &ms);
        if (rc && !rc_all) rc_all = rc;
        latency_ms[i] = std::chrono::duration<double, std::milli>(sub[(size_t)i] - due_of(i)).count() + ms;
    }
    submitter.join();
    if (elapsed_s) *elapsed_s = std::chrono::duration<double>(Clock::now() - t0).count();
    return sub_err ? sub_err.load() : rc_all;
}

MCGEN_API int mcgen_gb300_server_fail_next(McGb300Server *s, int code) {
    if (!s || code <= 0) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(s->m);
    s->fail_next = code;
    return MCGEN_OK;
}

MCGEN_API int mcgen_gb300_server_stats(McGb300Server *s, McGb300ServerStats *out) {
    if (!s || !out) return MCGEN_E_ARG;
    std::lock_guard<std::mutex> lk(s->m);
    *out = s->stats;
    out->pending = (long long)s->pending.size();
    long long used = 0;
    for (int d = 0; d < 3; d++) used += (long long)s->pool[d].map.size();
    out->cache_entries = used;
    return MCGEN_OK;
}

}  // extern "C"
