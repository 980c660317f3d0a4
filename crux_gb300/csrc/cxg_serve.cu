// Serving loop: continuous batching of likelihood and MC3-step requests.
//
// cxgServerSubmit copies a request (alignment patterns, tree, model) and
// returns a ticket at once.  A worker thread in the library runs the loop:
//
//   admit    while the request's device bytes fit the HBM budget and the
//            active-job limit: stream-ordered allocation (cudaMallocAsync,
//            so admission never synchronises the device; under memory
//            pressure the request waits in the queue), its op records
//            packed on the host into pinned staging and sent with one
//            copy, then the models of all admitted requests built on the
//            GPU in FP64 (Q eigensystem, Gamma categories, +I) by one
//            launch, a warp per request;
//   batch    every prepared lnL job joins the next persistent walker launch
//            (P matrices for all jobs, then (job, tile) items longest
//            first), one launch per number of mixture components; up to two
//            batches are in flight, so requests that arrive while one runs
//            are prepared and launched as soon as it retires;
//   retire   when a batch's event fires: read the lnLs, complete the
//            tickets (latency = submit to completion), free the memory.
//
// MC3-step requests run n generations of on-device MC3 (cxgMc3*) on four
// more workers; a session id keeps a chain resident across requests, and
// a session's requests run one at a time in submission order.  Their
// kernels run on their own streams and overlap the lnL batches.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "cxg_devmath.cuh"
#include "cxg_device.cuh"
#include "cxg_internal.h"

namespace cxg {

struct SrvModel {
    double rates[6], freqs[4], alpha, pinv;
    int32_t ncat, kact;
    double cube[64], eig[4], cmult[kMaxComps], rmult[kMaxComps];
    int32_t midx[kMaxComps];
    double wnorm;
    double pn[kMaxComps * 4];
    int32_t ok;
};

// Model of one request, FP64 on the GPU: mixture of ncat Gamma categories
// with weight (1 - pinv)/ncat each and, if pinv > 0, an invariant component
// (cmult 0) of weight pinv; wNorm and root weights as Lik.prep
// (Lik.pyx:1603-1665).  One warp per request (block b builds m[b]): lanes
// 0..ncat-2 compute the Gamma category cuts while lanes 28..31 form the
// eigensystem; lane 0 finishes.
constexpr unsigned kModelsPerLaunch = 128;
struct SrvModelList {
    SrvModel *m[kModelsPerLaunch];
};

__global__ void srv_model_kernel(SrvModelList list, unsigned n) {
    if (blockIdx.x >= n) return;
    SrvModel *m = list.m[blockIdx.x];
    __shared__ double tmp[74];
    __shared__ double cut[kMaxComps];
    __shared__ int bad;
    const unsigned lane = threadIdx.x;
    const int ncat = m->ncat;
    if (lane == 0) bad = 0;
    __syncwarp();
    if (ncat > 1 && (int)lane < ncat - 1) {
        const double c = d_gamma_cut(m->alpha, ncat, (int)lane);
        if (c == -1.0)
            bad = 1;
        else
            cut[lane] = c;
    }
    if (lane >= 28) qdecomp4_warp(m->rates, m->freqs, tmp, 28);
    __syncwarp();
    if (lane != 0) return;
    m->ok = 0;
    if (tmp[73] != 0.0 || bad) return;
    double pin[4];
    for (int i = 0; i < 4; ++i) pin[i] = tmp[i];
    const double qnorm = tmp[4];
    for (int i = 0; i < 64; ++i) m->cube[i] = tmp[5 + i];
    for (int i = 0; i < 4; ++i) m->eig[i] = tmp[69 + i];
    if (ncat > 1) {
        for (int i = 0; i + 1 < ncat; ++i) m->cmult[i] = cut[i];
        d_gamma_rates_from_cuts(ncat, m->cmult);
    } else {
        m->cmult[0] = 1.0;
    }
    double w[kMaxComps];
    for (int k = 0; k < ncat; ++k) w[k] = (1.0 - m->pinv) / ncat;
    int K = ncat;
    if (m->pinv > 0.0) {
        m->cmult[K] = 0.0;
        w[K] = m->pinv;
        ++K;
    }
    double qmean = 0.0;
    for (int k = 0; k < K; ++k) {
        m->rmult[k] = 1.0;
        m->midx[k] = 0;
        if (w[k] != 0.0 && m->cmult[k] != 0.0) qmean += w[k] * (1.0 / qnorm);
        for (int i = 0; i < 4; ++i) m->pn[k * 4 + i] = pin[i] * w[k];
    }
    m->wnorm = 1.0 / qmean;
    m->kact = K;
    m->ok = 1;
}

// Host plan of one likelihood request: post-order of the internal nodes,
// shared-memory stack slots, and which results must reach HBM (those a
// later op reads back from HBM because their slot was reused).
struct HostKid {
    int src;   // SRC_LEAF (idx = taxon), SRC_SLOT (idx = slot), SRC_GLOBAL
    int idx;   // ... or, for SRC_GLOBAL, the producer's HBM buffer index
    int node;  // child node (for its branch length)
};
struct HostPlan {
    bool ready = false;
    unsigned K = 0, ppad = 0, ntiles = 0, nops = 0, nk = 0, nslot = 0, nhbm = 0;
    unsigned tile = kTile, tpp = 1, ppt = 1, lmax = 0;
    bool staged = false;  // leaves staged per tile (else streamed)
    size_t rstride = 0, job_bytes = 0, data_bytes = 0;
    size_t up_bytes = 0;  // records .. model: the job's one upload
    std::vector<int> order, slot, hbm;
    std::vector<std::vector<HostKid>> kids;
};

// Patterns on the device: leaf masks, pattern weights and the table of the
// leaves' mask arrays (for jobs that stage their leaves).
// A registered dataset also keeps its host copy (MC3 requests build their
// chains from it) and a count of the admitted requests that use it.
struct SrvDataset {
    uint8_t *masks = nullptr;      // [ntaxa][ppad]
    uint32_t *weights = nullptr;   // [npat]
    const uint8_t **leaves = nullptr;  // [ntaxa] mask array of each taxon
    size_t stride = 0;  // mask row stride (>= the padded pattern count)
    char *mem = nullptr;
    size_t bytes = 0;
    unsigned ntaxa = 0, npat = 0;
    unsigned refs = 0;
    bool dropped = false;
    std::vector<uint8_t> hmasks;
    std::vector<uint32_t> hfreqs;
};

struct SrvRequest {
    uint64_t ticket = 0;
    HostPlan plan;
    SrvDataset *ds = nullptr;  // registered dataset (a reference is held)
    cxgRequest req;
    std::vector<uint8_t> masks;
    std::vector<uint32_t> pfreqs;
    std::vector<int32_t> parent;
    std::vector<double> len;
    std::chrono::steady_clock::time_point t_submit;
};

struct SrvResult {
    bool done = false;
    int rc = 0;
    double lnL = 0.0;
    double latency_ms = 0.0;
    std::string err;
};

struct SrvSession {
    cxgMc3 *mc3 = nullptr;
    size_t bytes = 0;
    uint64_t last_use = 0;
};

struct SrvJob {
    SrvDataset *ds = nullptr;       // resident patterns (cached or own)
    bool own_ds = false;
    std::unique_ptr<SrvRequest> rq;
    unsigned kact = 0, ppad = 0, ntiles = 0, nops = 0, nchild = 0;
    size_t bytes = 0;
    char *mem = nullptr;        // one stream-ordered allocation
    SrvModel *model = nullptr;  // in mem; built by srv_model_kernel
    PlanArgs a;
    PmatArgs pa;
    double updates = 0.0;
};

struct SrvBatch {
    std::vector<SrvJob *> jobs;
    char *mem = nullptr;  // jobs | items | pmat args | prefix | results
    size_t bytes = 0;
    cudaEvent_t done = nullptr;
    char *host = nullptr;  // pinned results (a slot of the server's pool)
    int slot = -1;
    cudaStream_t stream = nullptr;
};

// Pinned result slots, allocated once: no pinned allocation or release
// (which may synchronise) on the request path.
constexpr int kResultSlots = 8;

// Pinned upload staging.  The host writes a group's records, kid tables
// and models straight into pinned memory and sends each job with one copy;
// a copy from pageable memory may instead hold the calling thread until
// the stream drains.  A buffer is reused once the event recorded after its
// copies has completed; buffers grow (rarely: a pinned allocation may
// synchronise) to the largest group seen.  Used by the likelihood worker
// thread only.
constexpr unsigned kStageBufs = 16;
struct StageBuf {
    char *p = nullptr;
    size_t cap = 0;
    cudaEvent_t ev = nullptr;
    bool pending = false;
};
struct StagePool {
    std::vector<StageBuf> bufs;
    // A buffer of at least n bytes whose earlier copies are done, or null
    // on an allocation failure.
    StageBuf *get(size_t n) {
        if (bufs.capacity() < kStageBufs) bufs.reserve(kStageBufs);
        n = std::max<size_t>(n, 1);
        StageBuf *best = nullptr, *free_small = nullptr;
        for (auto &b : bufs) {
            if (b.pending && cudaEventQuery(b.ev) == cudaSuccess) b.pending = false;
            if (b.pending) continue;
            if (b.cap >= n && (!best || b.cap < best->cap)) best = &b;
            if (b.cap < n) free_small = &b;
        }
        if (best) return best;
        StageBuf *b = free_small;
        if (!b && bufs.size() < kStageBufs) {
            bufs.emplace_back();
            b = &bufs.back();
            if (cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) != cudaSuccess) {
                bufs.pop_back();
                return nullptr;
            }
        }
        if (!b) {  // all in flight: wait for the first
            b = &bufs.front();
            cudaEventSynchronize(b->ev);
            b->pending = false;
            if (b->cap >= n) return b;
        }
        if (b->p) host_free(b->p);
        b->p = nullptr;
        b->cap = 0;
        const size_t cap = std::max<size_t>(n, (size_t)1 << 20);
        if (host_alloc((void **)&b->p, cap) != cudaSuccess) return nullptr;
        b->cap = cap;
        return b;
    }
    // Mark b busy until the work now queued on s is done.
    void hand_off(StageBuf *b, cudaStream_t s) {
        cudaEventRecord(b->ev, s);
        b->pending = true;
    }
    void release() {
        for (auto &b : bufs) {
            if (b.pending) cudaEventSynchronize(b.ev);
            if (b.p) host_free(b.p);
            if (b.ev) cudaEventDestroy(b.ev);
        }
        bufs.clear();
    }
};

}  // namespace cxg

using namespace cxg;

struct cxgServer {
    cxgServerConfig cfg;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::unique_ptr<SrvRequest>> lnl_q, mc3_q;
    std::unordered_map<uint64_t, SrvResult> results;
    std::condition_variable done_cv;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;
    std::vector<std::thread> mc3_workers;
    std::unordered_set<uint64_t> mc3_busy;  // sessions a worker runs (under mu)
    unsigned mc3_running = 0;               // MC3 requests a worker runs (under mu)
    std::mutex sess_mu;                     // sessions, use_clock (before mu)
    cudaStream_t s_prep = nullptr, s_walk[2] = {nullptr, nullptr};
    size_t bytes_in_use = 0, bytes_peak = 0, budget = 0;
    std::vector<double> latencies;
    unsigned long long completed = 0, batches = 0, max_batch = 0, deferrals = 0;
    double updates_done = 0.0;
    std::chrono::steady_clock::time_point t_first, t_last;
    bool any_done = false;
    std::map<unsigned long long, SrvSession> sessions;
    uint64_t use_clock = 0;
    std::unordered_map<uint64_t, SrvDataset *> datasets;
    char *pinned = nullptr;  // [kResultSlots][max_active * 32]
    bool slot_busy[kResultSlots] = {};
    StagePool stage;  // likelihood worker's upload staging
};

namespace {

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t dataset_bytes(unsigned ntaxa, unsigned npat) {
    const size_t ppad = pad_patterns(npat);
    return al256((size_t)ntaxa * ppad) + al256((size_t)npat * 4) +
           al256((size_t)ntaxa * sizeof(void *));
}

// Plan a likelihood request on the host (no device work).
void plan_request(SrvRequest &rq, int prec) {
    HostPlan &P = rq.plan;
    const cxgRequest &r = rq.req;
    const unsigned N = r.ntaxa, NN = 2 * N - 2;
    P.K = r.ncat + (r.pinv > 0.0 ? 1 : 0);
    P.ppad = pad_patterns(r.npat);
    unsigned tq = 0;
    size_t budget = 0;
    unsigned pq = 1;
    cxgTuneGet(&P.tile, &tq, &pq, &budget);
    P.tpp = tuned_tpp(prec, P.K, P.tile);
    P.ppt = tuned_ppt(prec, P.K, P.tile, P.tpp);
    P.ntiles = P.ppad / P.tile;
    const size_t elt = prec == CXG_FP32 ? 4 : 8;
    const unsigned K = P.K;
    // Record stride: up to three children, each with the larger area (an
    // FP32 leaf's message table or a P matrix).
    P.rstride = (sizeof(RecHead) +
                 3 * (sizeof(RecChild) + std::max(child_area_bytes(prec, K, true),
                                                  child_area_bytes(prec, K, false))) +
                 15) & ~(size_t)15;
    std::vector<int32_t> child(NN * 3, -1);
    std::vector<int> nch(NN, 0);
    for (unsigned v = 0; v < NN; ++v) {
        const int pv = rq.parent[v];
        if (pv >= 0) child[pv * 3 + nch[pv]++] = (int)v;
    }
    P.order.clear();
    {
        std::vector<int> st{(int)r.root};
        while (!st.empty()) {
            const int v = st.back();
            st.pop_back();
            P.order.push_back(v);
            for (int j = 0; j < 3; ++j)
                if (child[v * 3 + j] >= (int)N) st.push_back(child[v * 3 + j]);
        }
        std::reverse(P.order.begin(), P.order.end());  // children first
    }
    const unsigned nops = (unsigned)P.order.size();
    // Leaf children per op (each op's mask rows travel with its record).
    P.lmax = 0;
    for (int v : P.order) {
        unsigned n = 0;
        for (int j = 0; j < 3; ++j) n += (child[v * 3 + j] >= 0 && child[v * 3 + j] < (int)N);
        if (n > P.lmax) P.lmax = n;
    }
    P.staged = (size_t)N * P.tile <= kLeafStageBytes;
    const unsigned s_lmax = P.staged ? 0 : P.lmax, s_nleaf = P.staged ? N : 0;
    const size_t base_b =
        plan_smem_bytes(prec, K, P.tile, 0, kRing, (unsigned)P.rstride, s_lmax, s_nleaf);
    const size_t slot_b =
        plan_smem_bytes(prec, K, P.tile, 1, kRing, (unsigned)P.rstride, s_lmax, s_nleaf) -
        base_b;
    unsigned cap = budget > base_b ? (unsigned)((budget - base_b) / slot_b) : 0;
    if (cap > kMaxSlots) cap = kMaxSlots;
    std::vector<int> owner(cap, -1), op_of(NN, -1);
    std::vector<char> need_hbm(nops, 0);
    P.slot.assign(nops, -1);
    P.kids.assign(nops, {});
    P.nslot = 0;
    P.nk = 0;
    for (unsigned o = 0; o < nops; ++o) {
        const int v = P.order[o];
        for (int j = 0; j < 3; ++j) {
            const int u = child[v * 3 + j];
            if (u < 0) continue;
            HostKid k;
            k.node = u;
            if (u < (int)N) {
                k.src = SRC_LEAF;
                k.idx = u;
            } else {
                const int prod = op_of[u];
                if (P.slot[prod] >= 0 && owner[P.slot[prod]] == prod) {
                    k.src = SRC_SLOT;
                    k.idx = P.slot[prod];
                    owner[P.slot[prod]] = -1;
                } else {
                    k.src = SRC_GLOBAL;
                    k.idx = prod;  // replaced by the HBM buffer index below
                    need_hbm[prod] = 1;
                }
            }
            P.kids[o].push_back(k);
            ++P.nk;
        }
        op_of[v] = (int)o;
        if (o + 1 < nops && cap > 0) {
            int sl = -1;
            for (unsigned q = 0; q < cap && sl < 0; ++q)
                if (owner[q] < 0) sl = (int)q;
            if (sl < 0) {
                int oldest = 0;
                for (unsigned q = 1; q < cap; ++q)
                    if (owner[q] < owner[oldest]) oldest = (int)q;
                sl = oldest;
            }
            owner[sl] = (int)o;
            P.slot[o] = sl;
            if ((unsigned)sl + 1 > P.nslot) P.nslot = sl + 1;
        }
    }
    P.hbm.assign(nops, -1);
    P.nhbm = 0;
    for (unsigned o = 0; o < nops; ++o)
        if (need_hbm[o]) P.hbm[o] = (int)P.nhbm++;
    for (auto &ks : P.kids)
        for (auto &k : ks)
            if (k.src == SRC_GLOBAL) k.idx = P.hbm[k.idx];
    P.nops = nops;
    const size_t kids = P.nk;
    size_t b = 0;
    b += al256((size_t)P.nhbm * K * 4 * P.ppad * elt);   // spilled CLs
    b += al256((size_t)P.nhbm * P.ppad * 8);             // their scalers
    b += al256((size_t)nops * P.rstride);                // records
    b += al256((size_t)nops * (P.lmax ? P.lmax : 1) * 8);  // leaf rows
    b += al256(kids * (8 + 8 + 4));                      // lens, dsts, tabs
    b += al256((size_t)P.ntiles * 16);                   // partial sums
    b += al256(sizeof(SrvModel));
    P.up_bytes = al256((size_t)nops * P.rstride) +
                 al256((size_t)nops * (P.lmax ? P.lmax : 1) * 8) + al256(kids * (8 + 8 + 4)) +
                 al256((size_t)P.ntiles * 16) + sizeof(SrvModel);
    if (prec == CXG_FP64) b += al256(kids * 16 * K * 4 * 8);
    P.job_bytes = b;
    P.data_bytes = dataset_bytes(N, r.npat);
    P.ready = true;
}

// Upload the patterns of a request into `ds` (one allocation on s).
int upload_dataset(unsigned N, unsigned npat, const uint8_t *masks,
                   const uint32_t *pfreqs, SrvDataset &ds, cudaStream_t s) {
    const size_t ppad = pad_patterns(npat);
    ds.bytes = dataset_bytes(N, npat);
    ds.ntaxa = N;
    ds.npat = npat;
    ds.stride = ppad;
    if (const cudaError_t e = dev_malloc_async((void **)&ds.mem, ds.bytes, s)) {
        ds.mem = nullptr;  // nothing for the caller to free
        return cuda_fail(e, "dev_malloc_async(server dataset)");
    }
    ds.masks = (uint8_t *)ds.mem;
    ds.weights = (uint32_t *)(ds.mem + al256((size_t)N * ppad));
    ds.leaves = (const uint8_t **)(ds.mem + al256((size_t)N * ppad) + al256((size_t)npat * 4));
    std::vector<uint8_t> hm((size_t)N * ppad, 15);
    for (unsigned t = 0; t < N; ++t) {
        const uint8_t *src = masks + (size_t)t * npat;
        uint8_t *dst = hm.data() + (size_t)t * ppad;
        for (unsigned q = 0; q < npat; ++q) {
            const uint8_t v = src[q] & 15;
            dst[q] = v ? v : 15;
        }
    }
    CXG_CUDA(cudaMemcpyAsync(ds.masks, hm.data(), hm.size(), cudaMemcpyHostToDevice, s));
    CXG_CUDA(cudaMemcpyAsync(ds.weights, pfreqs, (size_t)npat * 4,
                             cudaMemcpyHostToDevice, s));
    std::vector<const uint8_t *> hl(N);
    for (unsigned t = 0; t < N; ++t) hl[t] = ds.masks + (size_t)t * ppad;
    CXG_CUDA(cudaMemcpyAsync(ds.leaves, hl.data(), N * sizeof(void *),
                             cudaMemcpyHostToDevice, s));
    return 0;
}

// Device bytes of an MC3 session of `nc` chains (CLs dominate).
size_t mc3_bytes(const cxgRequest &r, int prec, unsigned nc) {
    const size_t elt = prec == CXG_FP32 ? 4 : 8;
    const size_t ppad = pad_patterns(r.npat), N = r.ntaxa, M = N - 2;
    const size_t K = r.ncat + (r.pinv > 0.0 ? 1 : 0);
    const size_t rstride =
        sizeof(RecHead) + 3 * (sizeof(RecChild) + std::max(child_area_bytes(prec, K, true),
                                                           child_area_bytes(prec, K, false))) +
        16;
    return nc * (2 * M * (K * 4 * ppad * elt + ppad * 8) + M * rstride) +
           N * ppad + ((size_t)4 << 20);
}

void complete(cxgServer *S, uint64_t ticket, int rc, double lnL,
              std::chrono::steady_clock::time_point t0) {
    const auto now = std::chrono::steady_clock::now();
    const std::string msg = rc ? std::string(cxgLastError()) : std::string();
    std::lock_guard<std::mutex> g(S->mu);
    SrvResult &r = S->results[ticket];
    r.done = true;
    r.rc = rc;
    r.err = msg;
    r.lnL = lnL;
    r.latency_ms = std::chrono::duration<double, std::milli>(now - t0).count();
    S->latencies.push_back(r.latency_ms);
    S->completed++;
    if (!S->any_done) S->t_first = now;
    S->any_done = true;
    S->t_last = now;
    S->done_cv.notify_all();
}

// Drop one reference to a registered dataset; returns it when it was the
// last one of a dropped dataset (the caller frees it).  Caller holds S->mu.
SrvDataset *unref_dataset(cxgServer *S, SrvDataset *ds) {
    if (ds == nullptr || --ds->refs != 0 || !ds->dropped) return nullptr;
    S->bytes_in_use -= ds->bytes;
    return ds;
}

// Give back what an lnL job holds: its memory and its dataset (its own
// copy, or its reference to a registered one).
void release_job(cxgServer *S, SrvJob *J, cudaStream_t st) {
    if (J->mem) dev_free_async(J->mem, st);
    SrvDataset *gone = nullptr;
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->bytes_in_use -= J->bytes;
        gone = J->own_ds ? J->ds : unref_dataset(S, J->ds);
    }
    if (gone) {
        if (gone->mem) dev_free_async(gone->mem, st);
        delete gone;
    }
    delete J;
}

// Returned by prepare_job when the job's memory cannot be had now: the
// request goes back to the head of the queue until batches in flight give
// their memory back.
constexpr int kDeferJob = 1;

// The device's stream-ordered pool keeps freed blocks, and a block freed
// on a batch stream may still be pending when the preparation stream asks
// for memory.  Wait for the streams and hand the pool's unused memory back
// so the next allocation can map it afresh.
void reclaim_pool(cxgServer *S) {
    for (auto &st : S->s_walk) cudaStreamSynchronize(st);
    cudaStreamSynchronize(S->s_prep);
    int dev = 0;
    cudaMemPool_t pool = nullptr;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetMemPool(&pool, dev) == cudaSuccess) {
        std::lock_guard<std::mutex> gate(capture_gate());  // unmaps device memory
        cudaMemPoolTrimTo(pool, 0);
    }
}

// Prepare an admitted lnL request: upload its patterns unless they are a
// registered dataset, allocate its job memory, write its records, kid
// tables and model parameters into `stage` (pinned, plan.up_bytes, laid
// out as the job memory from the records to the model) and send them with
// one copy.  The model itself is built by srv_model_kernel afterwards.
int prepare_job(cxgServer *S, SrvJob &J, char *stage) {
    const cxgRequest &r = J.rq->req;
    const HostPlan &P = J.rq->plan;
    const int prec = S->cfg.precision;
    const unsigned N = r.ntaxa;
    if (J.rq->ds) {
        J.ds = J.rq->ds;
    } else {
        J.ds = new SrvDataset();
        J.own_ds = true;
        const int rc = upload_dataset(N, r.npat, J.rq->masks.data(), J.rq->pfreqs.data(),
                                      *J.ds, S->s_prep);
        if (rc) return rc;
    }
    const unsigned K = P.K;
    const size_t elt = prec == CXG_FP32 ? 4 : 8;
    const size_t ppad = P.ppad, rstride = P.rstride;
    J.kact = K;
    J.ppad = P.ppad;
    J.ntiles = P.ntiles;
    cudaError_t ae = dev_malloc_async((void **)&J.mem, P.job_bytes, S->s_prep);
    if (ae == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        reclaim_pool(S);
        ae = dev_malloc_async((void **)&J.mem, P.job_bytes, S->s_prep);
    }
    if (ae == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        J.mem = nullptr;
        return kDeferJob;
    }
    if (ae != cudaSuccess) {
        J.mem = nullptr;
        return cuda_fail(ae, "dev_malloc_async(server job)");
    }
    char *p = J.mem;
    auto take = [&](size_t n) {
        char *q = p;
        p += al256(n);
        return q;
    };
    char *cls = take((size_t)P.nhbm * K * 4 * ppad * elt);
    char *scs = take((size_t)P.nhbm * ppad * 8);
    unsigned char *rec = (unsigned char *)take((size_t)P.nops * rstride);
    const uint8_t **lrows =
        (const uint8_t **)take((size_t)P.nops * (P.lmax ? P.lmax : 1) * sizeof(void *));
    char *kidarr = take((size_t)P.nk * (8 + 8 + 4));
    double *partial = (double *)take((size_t)P.ntiles * 16);
    SrvModel *model = (SrvModel *)take(sizeof(SrvModel));
    double *ltab = prec == CXG_FP64 ? (double *)take((size_t)P.nk * 16 * K * 4 * 8) : nullptr;
    double *klen = (double *)kidarr;
    uint64_t *kdst = (uint64_t *)(kidarr + (size_t)P.nk * 8);
    int32_t *ktab = (int32_t *)(kidarr + (size_t)P.nk * 16);
    auto cl_of = [&](int h) { return cls + (size_t)h * K * 4 * ppad * elt; };
    auto sc_of = [&](int h) { return scs + (size_t)h * ppad * 8; };
    // Host images at the same offsets from `stage` as on the device from rec.
    auto host_of = [&](const void *d) {
        return stage + ((const char *)d - (const char *)rec);
    };
    unsigned char *hrec = (unsigned char *)stage;
    const uint8_t **hlr = (const uint8_t **)host_of(lrows);
    double *hlen = (double *)host_of(klen);
    uint64_t *hdst = (uint64_t *)host_of(kdst);
    int32_t *htab = (int32_t *)host_of(ktab);
    memset(hrec, 0, (size_t)P.nops * rstride);
    memset(hlr, 0, (size_t)P.nops * (P.lmax ? P.lmax : 1) * sizeof(void *));
    for (unsigned i = 0; i < P.nk; ++i) htab[i] = -1;
    unsigned nk = 0;
    for (unsigned o = 0; o < P.nops; ++o) {
        unsigned char *rr = hrec + (size_t)o * rstride;
        const unsigned nch = (unsigned)P.kids[o].size();
        RecHead hd;
        memset(&hd, 0, sizeof(hd));
        hd.nchild = nch;
        hd.slot = P.slot[o];
        if (P.hbm[o] >= 0) {
            hd.data = cl_of(P.hbm[o]);
            hd.scaler = sc_of(P.hbm[o]);
        } else {
            hd.flags = REC_NO_HBM;
        }
        memcpy(rr, &hd, sizeof(hd));
        size_t area = sizeof(RecHead) + nch * sizeof(RecChild);
        int kcls[3] = {1, 1, 1};
        for (unsigned ci = 0; ci < nch; ++ci) {
            const HostKid &k = P.kids[o][ci];
            RecChild ch;
            memset(&ch, 0, sizeof(ch));
            ch.src = (uint32_t)k.src;
            ch.off = (uint32_t)area;
            if (k.src == SRC_LEAF) {
                ch.data = J.ds->masks + (size_t)k.idx * J.ds->stride;  // taxon's masks
                ch.idx = (uint32_t)k.idx;                       // its staged row
                const uint8_t **lr = hlr + (size_t)o * P.lmax;
                unsigned j = 0;
                while (lr[j] != nullptr) ++j;
                lr[j] = static_cast<const uint8_t *>(ch.data);
                ch.tab = prec == CXG_FP64 ? nk : 0;
                htab[nk] = prec == CXG_FP64 ? (int32_t)nk : 0;
            } else if (k.src == SRC_SLOT) {
                ch.idx = (uint32_t)k.idx;
            } else {
                ch.data = cl_of(k.idx);
                ch.scaler = sc_of(k.idx);
            }
            memcpy(rr + sizeof(RecHead) + ci * sizeof(RecChild), &ch, sizeof(ch));
            // Class for the op kind: the previous op's node is F (its result
            // is still in the walker's registers).
            kcls[ci] = k.src == SRC_LEAF ? 0 : (o > 0 && k.node == P.order[o - 1] ? 2 : 1);
            hlen[nk] = J.rq->len[k.node];
            hdst[nk] = (size_t)o * rstride + area;
            area += child_area_bytes(prec, K, k.src == SRC_LEAF);
            ++nk;
        }
        if (prec == CXG_FP32 && nch == 2) {
            hd.flags |= op_kind_of_classes(kcls[0], kcls[1]);
            memcpy(rr, &hd, sizeof(hd));
        }
    }
    SrvModel &hmod = *(SrvModel *)host_of(model);
    memset(&hmod, 0, sizeof(hmod));
    memcpy(hmod.rates, r.rates, 48);
    memcpy(hmod.freqs, r.freqs, 32);
    hmod.alpha = r.alpha;
    hmod.pinv = r.pinv;
    hmod.ncat = (int32_t)r.ncat;
    // The partial sums between the kid tables and the model go up too
    // (unset; the walker writes them before it reads them).
    CXG_CUDA(cudaMemcpyAsync(rec, stage, P.up_bytes, cudaMemcpyHostToDevice, S->s_prep));
    J.model = model;

    PlanArgs &a = J.a;
    memset(&a, 0, sizeof(a));
    a.rec = rec;
    a.lrows = lrows;
    a.lmax = P.staged ? 0 : P.lmax;
    a.leaves = P.staged ? J.ds->leaves : nullptr;
    a.nleaf = P.staged ? N : 0;
    a.rstride = (uint32_t)rstride;
    a.ring = kRing;
    a.nops = P.nops;
    a.nslot = P.nslot;
    a.tile = P.tile;
    a.tpp = P.tpp;
    a.ppt = P.ppt;
    a.kact = K;
    a.npat = r.npat;
    a.ppad = J.ppad;
    a.root_last = 1;
    a.pn = model->pn;
    a.freqs = J.ds->weights;
    a.partial = partial;
    a.ltab = ltab;
    a.ntiles = J.ntiles;
    PmatArgs &pa = J.pa;
    pa = PmatArgs{};
    pa.nchild = nk;
    pa.kact = K;
    pa.precision = prec;
    pa.edge_len = klen;
    pa.cmult = model->cmult;
    pa.rmult = model->rmult;
    pa.model = model->midx;
    pa.cube = model->cube;
    pa.eig = model->eig;
    pa.dst = kdst;
    pa.tab = ktab;
    pa.wnorm_dev = &model->wnorm;
    pa.rec = rec;
    pa.ltab = ltab;
    J.nops = P.nops;
    J.nchild = nk;
    J.updates = (double)J.nops * r.npat;
    return 0;
}

// Launch one batch of prepared jobs (all of one walker shape).
int launch_batch_of(cxgServer *S, SrvBatch &B, cudaStream_t st) {
    NvtxRange nr("cxgServer batch launch");
    const size_t n = B.jobs.size();
    std::vector<PlanArgs> jobs(n);
    std::vector<PmatArgs> pm(n);
    std::vector<uint32_t> prefix(n + 1, 0);
    std::vector<WalkItem> items;
    unsigned max_nslot = 0, max_rstride = 16, max_lmax = 0, max_nleaf = 0;
    size_t nitems = 0;
    for (size_t j = 0; j < n; ++j) nitems += B.jobs[j]->ntiles;
    const size_t o_jobs = 0, o_items = al256(n * sizeof(PlanArgs));
    const size_t o_pm = o_items + al256(nitems * sizeof(WalkItem));
    const size_t o_pre = o_pm + al256(n * sizeof(PmatArgs));
    const size_t o_res = o_pre + al256((n + 1) * 4);
    B.bytes = o_res + al256(n * 32 + 16);
    B.slot = -1;
    for (int k = 0; k < kResultSlots && B.slot < 0; ++k)
        if (!S->slot_busy[k]) B.slot = k;
    if (B.slot < 0) return fail(CXG_EBUSY, "server: no free result slot");
    S->slot_busy[B.slot] = true;
    B.host = S->pinned + (size_t)B.slot * S->cfg.max_active * 32;
    if (const cudaError_t e = dev_malloc_async((void **)&B.mem, B.bytes, st)) {
        B.mem = nullptr;
        return cuda_fail(e, "dev_malloc_async(server batch)");
    }
    char *res = B.mem + o_res;
    for (size_t j = 0; j < n; ++j) {
        SrvJob *J = B.jobs[j];
        PlanArgs a = J->a;
        a.ticket = (unsigned *)(res + j * 32);
        a.ninf = (uint32_t *)(res + j * 32 + 4);
        a.err = (uint32_t *)(res + j * 32 + 8);
        a.total = (double *)(res + j * 32 + 16);
        jobs[j] = a;
        pm[j] = J->pa;
        prefix[j + 1] = prefix[j] + J->nchild * J->kact;
        for (unsigned t = 0; t < J->ntiles; ++t) items.push_back(WalkItem{(uint32_t)j, t});
        max_nslot = std::max(max_nslot, a.nslot);
        max_rstride = std::max(max_rstride, a.rstride);
        max_lmax = std::max(max_lmax, a.lmax);
        max_nleaf = std::max(max_nleaf, a.nleaf);
    }
    std::stable_sort(items.begin(), items.end(), [&](const WalkItem &x, const WalkItem &y) {
        return jobs[x.job].nops > jobs[y.job].nops;
    });
    StageBuf *sb = S->stage.get(o_res);
    if (!sb) return fail(CXG_ENOMEM, "server: pinned staging");
    char *host = sb->p;
    memcpy(host + o_jobs, jobs.data(), n * sizeof(PlanArgs));
    memcpy(host + o_items, items.data(), items.size() * sizeof(WalkItem));
    memcpy(host + o_pm, pm.data(), n * sizeof(PmatArgs));
    memcpy(host + o_pre, prefix.data(), (n + 1) * 4);
    const cudaError_t ce = cudaMemcpyAsync(B.mem, host, o_res, cudaMemcpyHostToDevice, st);
    S->stage.hand_off(sb, st);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(server batch)");
    CXG_CUDA(cudaMemsetAsync(res, 0, n * 32 + 16, st));
    CXG_CUDA(launch_pmat_batch((const PmatArgs *)(B.mem + o_pm),
                               (const uint32_t *)(B.mem + o_pre), (uint32_t)n,
                               prefix[n], st));
    BatchArgs ba{};
    ba.jobs = (const PlanArgs *)(B.mem + o_jobs);
    ba.items = (const WalkItem *)(B.mem + o_items);
    ba.nitems = (uint32_t)items.size();
    ba.counter = (unsigned *)(res + n * 32);
    ba.tile = B.jobs[0]->a.tile;
    ba.tpp = B.jobs[0]->a.tpp;
    ba.ppt = B.jobs[0]->a.ppt;
    ba.ring = kRing;
    ba.kact = B.jobs[0]->kact;
    ba.max_nslot = max_nslot;
    ba.max_rstride = max_rstride;
    ba.max_lmax = max_lmax;
    ba.max_nleaf = max_nleaf;
    const int prec = S->cfg.precision;
    const size_t smem = plan_smem_bytes(prec, ba.kact, ba.tile, max_nslot,
                                        kRing, max_rstride, max_lmax, max_nleaf);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int per =
        batch_ctas_per_sm(prec, ba.kact, ba.tile, ba.tpp, ba.ppt, max_lmax == 0, smem);
    if (per <= 0) return fail(CXG_EINVAL, "server: walker does not fit an SM");
    cudaError_t e = launch_batch(prec, ba, (unsigned)(per * nsm), st);
    if (e != cudaSuccess) return cuda_fail(e, "walk_batch_kernel (server)");
    CXG_CUDA(cudaMemcpyAsync(B.host, res, n * 32, cudaMemcpyDeviceToHost, st));
    CXG_CUDA(cudaEventCreateWithFlags(&B.done, cudaEventDisableTiming));
    CXG_CUDA(cudaEventRecord(B.done, st));
    B.stream = st;
    return 0;
}

void retire(cxgServer *S, SrvBatch &B) {
    const size_t n = B.jobs.size();
    for (size_t j = 0; j < n; ++j) {
        SrvJob *J = B.jobs[j];
        uint32_t ninf, err;
        double tot[2];
        memcpy(&ninf, B.host + j * 32 + 4, 4);
        memcpy(&err, B.host + j * 32 + 8, 4);
        memcpy(tot, B.host + j * 32 + 16, 16);
        const double v = ninf ? -INFINITY : tot[0] + tot[1];
        if (err) fail(CXG_ETIMEOUT, "walk_batch_kernel (server): record wait timed out");
        complete(S, J->rq->ticket, err ? CXG_ETIMEOUT : 0, v, J->rq->t_submit);
        {
            std::lock_guard<std::mutex> g(S->mu);
            S->updates_done += J->updates;
        }
        release_job(S, J, B.stream);
    }
    dev_free_async(B.mem, B.stream);
    cudaEventDestroy(B.done);
    S->slot_busy[B.slot] = false;
}

// Evict the least recently used MC3 session that no worker runs; the
// caller holds sess_mu.  False if every session is in use (or none).
bool evict_lru_session(cxgServer *S) {
    auto lru = S->sessions.end();
    {
        std::lock_guard<std::mutex> g(S->mu);
        for (auto q = S->sessions.begin(); q != S->sessions.end(); ++q)
            if (!S->mc3_busy.count(q->first) &&
                (lru == S->sessions.end() || q->second.last_use < lru->second.last_use))
                lru = q;
        if (lru == S->sessions.end()) return false;
        S->bytes_in_use -= lru->second.bytes;
    }
    cxgMc3Destroy(lru->second.mc3);
    S->sessions.erase(lru);
    return true;
}

void lnl_loop(cxgServer *S) {
    std::vector<SrvJob *> ready;        // prepared, waiting for a batch
    std::deque<SrvBatch> inflight;
    cudaEvent_t prep_done = nullptr;
    cudaEventCreateWithFlags(&prep_done, cudaEventDisableTiming);
    unsigned next_stream = 0;
    for (;;) {
        // 1. Admit.
        std::vector<SrvJob *> admitted;
        bool blocked = false;  // the head does not fit and no lnL job holds memory
        {
            std::unique_lock<std::mutex> g(S->mu);
            if (S->lnl_q.empty() && ready.empty() && inflight.empty()) {
                if (S->stop) break;
                S->cv.wait_for(g, std::chrono::milliseconds(2));
                if (S->stop && S->lnl_q.empty()) break;
            }
            const size_t active = ready.size() + [&] {
                size_t c = 0;
                for (auto &b : inflight) c += b.jobs.size();
                return c;
            }();
            while (!S->lnl_q.empty() && active + admitted.size() < S->cfg.max_active) {
                SrvRequest &rq = *S->lnl_q.front();
                const size_t need = rq.plan.job_bytes + (rq.ds ? 0 : rq.plan.data_bytes);
                if (S->bytes_in_use + need > S->budget && S->bytes_in_use > 0) {
                    blocked = active == 0 && admitted.empty();
                    break;
                }
                SrvJob *J = new SrvJob();
                J->bytes = need;
                J->rq = std::move(S->lnl_q.front());
                S->lnl_q.pop_front();
                S->bytes_in_use += need;
                S->bytes_peak = std::max(S->bytes_peak, S->bytes_in_use);
                admitted.push_back(J);
            }
        }
        // Only idle MC3 sessions (and resident datasets) hold the budget:
        // give the head request the memory of the least recently used one.
        if (blocked) {
            bool freed;
            {
                std::lock_guard<std::mutex> sg(S->sess_mu);
                freed = evict_lru_session(S);
            }
            if (!freed) {
                // Closing with no MC3 request left to give memory back:
                // the request fails rather than hold the close up.
                std::unique_ptr<SrvRequest> gone;
                SrvDataset *gds = nullptr;
                {
                    std::lock_guard<std::mutex> g(S->mu);
                    if (S->stop && S->mc3_running == 0 && !S->lnl_q.empty()) {
                        gone = std::move(S->lnl_q.front());
                        S->lnl_q.pop_front();
                        gds = unref_dataset(S, gone->ds);
                    }
                }
                if (gone) {
                    complete(S, gone->ticket,
                             fail(CXG_ENOMEM, "server closed before the request's memory "
                                              "was free"),
                             NAN, gone->t_submit);
                    if (gds) {
                        dev_free(gds->mem);
                        delete gds;
                    }
                } else {
                    // Sessions in use give their memory back when they finish.
                    std::this_thread::sleep_for(std::chrono::microseconds(200));
                }
            }
        }
        if (!admitted.empty()) {
            NvtxRange nr("cxgServer prepare");
            size_t up = 0;
            for (SrvJob *J : admitted) up += al256(J->rq->plan.up_bytes);
            StageBuf *sb = S->stage.get(up);
            char *hp = sb ? sb->p : nullptr;
            std::vector<SrvJob *> prepared;
            std::vector<std::unique_ptr<SrvRequest>> deferred;
            for (SrvJob *J : admitted) {
                int rc = !deferred.empty() ? kDeferJob
                         : sb             ? prepare_job(S, *J, hp)
                                          : fail(CXG_ENOMEM, "server: pinned staging");
                if (hp) hp += al256(J->rq->plan.up_bytes);
                // Out of memory with nothing else holding any: a failure.
                if (rc == kDeferJob && deferred.empty() && prepared.empty() &&
                    ready.empty() && inflight.empty())
                    rc = fail(CXG_ENOMEM, "server: job memory (cudaMallocAsync)");
                if (rc == kDeferJob) {
                    if (J->mem) dev_free_async(J->mem, S->s_prep);
                    if (J->own_ds && J->ds) {
                        if (J->ds->mem) dev_free_async(J->ds->mem, S->s_prep);
                        delete J->ds;
                    }
                    {
                        std::lock_guard<std::mutex> g(S->mu);
                        S->bytes_in_use -= J->bytes;
                    }
                    deferred.push_back(std::move(J->rq));
                    delete J;
                    continue;
                }
                if (rc) {
                    complete(S, J->rq->ticket, rc, NAN, J->rq->t_submit);
                    release_job(S, J, S->s_prep);
                    continue;
                }
                prepared.push_back(J);
            }
            // One model launch per kModelsPerLaunch jobs, a warp per job.
            for (size_t i = 0; i < prepared.size(); i += kModelsPerLaunch) {
                const unsigned nm =
                    (unsigned)std::min<size_t>(kModelsPerLaunch, prepared.size() - i);
                SrvModelList ml;
                for (unsigned j = 0; j < nm; ++j) ml.m[j] = prepared[i + j]->model;
                srv_model_kernel<<<nm, 32, 0, S->s_prep>>>(ml, nm);
                const cudaError_t e = cudaGetLastError();
                for (unsigned j = 0; j < nm; ++j) {
                    SrvJob *J = prepared[i + j];
                    if (e == cudaSuccess) {
                        ready.push_back(J);
                        continue;
                    }
                    complete(S, J->rq->ticket, cuda_fail(e, "srv_model_kernel"), NAN,
                             J->rq->t_submit);
                    release_job(S, J, S->s_prep);
                }
            }
            if (sb) S->stage.hand_off(sb, S->s_prep);
            if (!deferred.empty()) {
                std::lock_guard<std::mutex> g(S->mu);
                for (size_t i = deferred.size(); i-- > 0;)
                    S->lnl_q.push_front(std::move(deferred[i]));
                S->deferrals += deferred.size();
            }
            cudaEventRecord(prep_done, S->s_prep);
            // Batch streams wait for the preparation of these jobs.
            for (auto &st : S->s_walk) cudaStreamWaitEvent(st, prep_done, 0);
        }
        // 2. Retire finished batches.
        while (!inflight.empty() && cudaEventQuery(inflight.front().done) == cudaSuccess) {
            retire(S, inflight.front());
            inflight.pop_front();
        }
        // 3. Launch a batch per component count while a stream is free.
        if (!ready.empty() && inflight.size() < 2) {
            // A failed launch must give its slot back.
            // One launch per walker shape: components, tile, threads per
            // pattern, staged or streamed leaves.
            std::map<unsigned, std::vector<SrvJob *>> byk;
            for (SrvJob *J : ready)
                byk[J->kact | J->a.tile << 8 | J->a.tpp << 16 | J->a.ppt << 20 |
                    (J->a.lmax ? 1u : 0u) << 24]
                    .push_back(J);
            ready.clear();
            for (auto &kv : byk) {
                SrvBatch B;
                B.jobs = kv.second;
                cudaStream_t st = S->s_walk[next_stream++ % 2];
                const int rc = launch_batch_of(S, B, st);
                if (rc && B.slot >= 0) S->slot_busy[B.slot] = false;
                if (rc) {
                    if (B.mem) dev_free_async(B.mem, st);
                    if (B.done) cudaEventDestroy(B.done);
                    for (SrvJob *J : B.jobs) {
                        complete(S, J->rq->ticket, rc, NAN, J->rq->t_submit);
                        release_job(S, J, st);
                    }
                    continue;
                }
                {
                    std::lock_guard<std::mutex> g(S->mu);
                    S->batches++;
                    S->max_batch = std::max<unsigned long long>(S->max_batch, B.jobs.size());
                }
                inflight.push_back(B);
            }
        } else if (!inflight.empty()) {
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
    for (auto &b : inflight) {
        cudaEventSynchronize(b.done);
        retire(S, b);
    }
    cudaEventDestroy(prep_done);
}

// MC3 requests run on kMc3Workers threads, each session's handle (own
// stream and generation graph) on one of them at a time: small sessions
// overlap on the device, and the requests of a session keep their order.
constexpr unsigned kMc3Workers = 4;

void mc3_loop(cxgServer *S) {
    for (;;) {
        std::unique_ptr<SrvRequest> rq;
        {
            std::unique_lock<std::mutex> g(S->mu);
            // The first queued request whose session no other worker runs.
            auto runnable = [&] {
                for (auto q = S->mc3_q.begin(); q != S->mc3_q.end(); ++q)
                    if ((*q)->req.session == 0 || !S->mc3_busy.count((*q)->req.session))
                        return q;
                return S->mc3_q.end();
            };
            S->cv.wait_for(g, std::chrono::milliseconds(2), [&] {
                return runnable() != S->mc3_q.end() || (S->stop && S->mc3_q.empty());
            });
            auto q = runnable();
            if (q == S->mc3_q.end()) {
                if (S->stop && S->mc3_q.empty()) break;
                continue;
            }
            rq = std::move(*q);
            S->mc3_q.erase(q);
            if (rq->req.session) S->mc3_busy.insert(rq->req.session);
            ++S->mc3_running;
        }
        const cxgRequest &r = rq->req;
        cxgMc3 *m = nullptr;
        int rc = 0;
        const unsigned nc = r.mc3_chains ? r.mc3_chains : 4;
        const size_t need = mc3_bytes(r, S->cfg.precision, nc);
        {
            std::lock_guard<std::mutex> sg(S->sess_mu);
            auto it = r.session ? S->sessions.find(r.session) : S->sessions.end();
            if (it != S->sessions.end()) {
                m = it->second.mc3;
                it->second.last_use = ++S->use_clock;
            } else {
                // Admission by free HBM: evict idle sessions (none that a
                // worker runs), least recently used first, until the new
                // chains fit the budget.
                for (;;) {
                    bool fits;
                    {
                        std::lock_guard<std::mutex> g(S->mu);
                        fits = S->bytes_in_use + need <= S->budget;
                    }
                    if (fits || !evict_lru_session(S)) {  // (or nothing to evict)
                        std::lock_guard<std::mutex> g(S->mu);
                        S->bytes_in_use += need;
                        S->bytes_peak = std::max(S->bytes_peak, S->bytes_in_use);
                        break;
                    }
                }
            }
        }
        if (m == nullptr) {
            cxgMc3Config c;
            memset(&c, 0, sizeof(c));
            c.ntaxa = r.ntaxa;
            c.npat = r.npat;
            c.masks = rq->ds ? rq->ds->hmasks.data() : rq->masks.data();
            c.freqs_pattern = rq->ds ? rq->ds->hfreqs.data() : rq->pfreqs.data();
            c.parent = rq->parent.data();
            c.len = rq->len.data();
            c.root = r.root;
            memcpy(c.rates, r.rates, 48);
            memcpy(c.freqs, r.freqs, 32);
            c.alpha = r.alpha;
            c.ncat = r.ncat;
            c.nchains = nc;
            c.heat_delta = r.mc3_heat_delta > 0.0 ? r.mc3_heat_delta : 0.1;
            c.swap_stride = 1;
            c.seed = r.seed;
            c.move_weight[0] = 1.0;
            c.move_weight[1] = 1.0;
            c.brlen_lambda = 2.0 * log(1.6);
            c.brlen_prior = 10.0;
            c.rate_conc = 300.0;
            c.alpha_lambda = 2.0 * log(1.6);
            c.alpha_prior = 1.0;
            c.pinv = r.pinv;
            c.invar_lambda = 2.0 * log(1.6);
            c.invar_prior = 0.5;
            c.gamma_jump_prior = 1.0;
            c.freq_jump_prior = 1.0;
            c.invar_jump_prior = 1.0;
            for (int i = 0; i < 6; ++i) c.rclass[i] = i;
            c.rate_jump_prior = 1.0;
            c.rate_lambda = 2.0 * log(1.6);
            c.precision = S->cfg.precision;
            c.graph_gens = r.mc3_gens ? r.mc3_gens : 10;
            c.trace_cap = 1;
            rc = cxgMc3Create(&c, &m);
            if (rc == 0 && r.session) {
                std::lock_guard<std::mutex> sg(S->sess_mu);
                SrvSession ss;
                ss.mc3 = m;
                ss.bytes = need;
                ss.last_use = ++S->use_clock;
                S->sessions[r.session] = ss;
            } else {
                std::lock_guard<std::mutex> g(S->mu);
                S->bytes_in_use -= need;
            }
        }
        double lnl = NAN;
        if (rc == 0) rc = cxgMc3Run(m, r.mc3_gens ? r.mc3_gens : 10, nullptr);
        if (rc == 0) rc = mc3_cold_lnl(m, &lnl);  // the cold chain's
        if (m && !r.session) cxgMc3Destroy(m);
        complete(S, rq->ticket, rc, lnl, rq->t_submit);
        SrvDataset *gone = nullptr;
        {
            std::lock_guard<std::mutex> g(S->mu);
            gone = unref_dataset(S, rq->ds);
            if (r.session) S->mc3_busy.erase(r.session);
            --S->mc3_running;
        }
        S->cv.notify_all();  // a worker may wait for this session
        if (gone) {
            dev_free(gone->mem);
            delete gone;
        }
    }
}

}  // namespace

extern "C" int cxgServerCreate(const cxgServerConfig *cfg, cxgServer **out) {
    if (cfg == nullptr || out == nullptr) return fail(CXG_EINVAL, "cxgServerCreate: NULL");
    if (cfg->precision != CXG_FP32 && cfg->precision != CXG_FP64)
        return fail(CXG_EINVAL, "cxgServerCreate: unknown precision");
    cxgServer *S = new cxgServer();
    S->cfg = *cfg;
    if (S->cfg.max_active == 0) S->cfg.max_active = 256;
    size_t fr = 0, tot = 0;
    cudaError_t e = cudaMemGetInfo(&fr, &tot);
    if (e != cudaSuccess) {
        delete S;
        return cuda_fail(e, "cudaMemGetInfo");
    }
    S->budget = cfg->hbm_budget ? (size_t)cfg->hbm_budget : (size_t)(fr * 0.8);
    if ((e = host_alloc((void **)&S->pinned,
                        (size_t)kResultSlots * S->cfg.max_active * 32)) != cudaSuccess) {
        delete S;
        return cuda_fail(e, "cudaHostAlloc(server results)");
    }
    if ((e = cudaStreamCreateWithFlags(&S->s_prep, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&S->s_walk[0], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&S->s_walk[1], cudaStreamNonBlocking)) != cudaSuccess) {
        delete S;
        return cuda_fail(e, "cudaStreamCreate(server)");
    }
    int dev = 0;
    cudaGetDevice(&dev);
    S->worker = std::thread([S, dev] {
        cudaSetDevice(dev);
        lnl_loop(S);
    });
    for (unsigned w = 0; w < kMc3Workers; ++w)
        S->mc3_workers.emplace_back([S, dev] {
            cudaSetDevice(dev);
            mc3_loop(S);
        });
    *out = S;
    return 0;
}

extern "C" int cxgServerSubmit(cxgServer *S, const cxgRequest *r,
                               unsigned long long *ticket) {
    if (S == nullptr || r == nullptr || ticket == nullptr)
        return fail(CXG_EINVAL, "cxgServerSubmit: NULL");
    if (r->ntaxa < 3 || r->npat == 0 || r->ncat < 1 ||
        r->ncat + (r->pinv > 0.0 ? 1 : 0) > kMaxComps)
        return fail(CXG_EINVAL, "cxgServerSubmit: bad request shape");
    if (r->kind != CXG_REQ_LNL && r->kind != CXG_REQ_MC3)
        return fail(CXG_EINVAL, "cxgServerSubmit: unknown request kind");
    const unsigned N = r->ntaxa, NN = 2 * N - 2;
    if (r->root < N || r->root >= NN) return fail(CXG_EINVAL, "cxgServerSubmit: bad root");
    std::vector<int> nch(NN, 0);
    for (unsigned v = 0; v < NN; ++v) {
        const int p = r->parent[v];
        if (v == r->root ? p != -1 : (p < (int)N || p >= (int)NN))
            return fail(CXG_EINVAL, "cxgServerSubmit: bad parent array");
        if (p >= 0 && ++nch[p] > 3) return fail(CXG_EINVAL, "cxgServerSubmit: degree > 3");
    }
    for (unsigned v = N; v < NN; ++v)
        if (nch[v] != (v == r->root ? 3 : 2))
            return fail(CXG_EINVAL, "cxgServerSubmit: tree is not binary");
    auto rq = std::make_unique<SrvRequest>();
    rq->req = *r;
    if (r->dataset == 0) {
        if (r->masks == nullptr || r->pattern_freqs == nullptr)
            return fail(CXG_EINVAL, "cxgServerSubmit: no patterns");
        rq->masks.assign(r->masks, r->masks + (size_t)r->ntaxa * r->npat);
        rq->pfreqs.assign(r->pattern_freqs, r->pattern_freqs + r->npat);
    }
    rq->parent.assign(r->parent, r->parent + NN);
    rq->len.assign(r->len, r->len + NN);
    rq->req.masks = nullptr;
    rq->req.pattern_freqs = nullptr;
    rq->req.parent = nullptr;
    rq->req.len = nullptr;
    // Plan on the submitting thread: admission then charges exact bytes.
    if (r->kind == CXG_REQ_LNL) plan_request(*rq, S->cfg.precision);
    rq->t_submit = std::chrono::steady_clock::now();
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (r->dataset) {
            auto it = S->datasets.find(r->dataset);
            if (it == S->datasets.end())
                return fail(CXG_EINVAL, "cxgServerSubmit: unknown dataset");
            SrvDataset *ds = it->second;
            if (ds->ntaxa != r->ntaxa || ds->npat != r->npat)
                return fail(CXG_EINVAL, "cxgServerSubmit: request shape differs from its dataset");
            ds->refs++;
            rq->ds = ds;
        }
        rq->ticket = S->next_ticket++;
        *ticket = rq->ticket;
        S->results[rq->ticket] = SrvResult();
        if (r->kind == CXG_REQ_LNL)
            S->lnl_q.push_back(std::move(rq));
        else
            S->mc3_q.push_back(std::move(rq));
    }
    S->cv.notify_all();
    return 0;
}

extern "C" int cxgServerWait(cxgServer *S, unsigned long long ticket, double timeout_s,
                             double *lnL, double *latency_ms) {
    if (S == nullptr) return fail(CXG_EINVAL, "cxgServerWait: NULL");
    std::unique_lock<std::mutex> g(S->mu);
    auto it = S->results.find(ticket);
    if (it == S->results.end()) return fail(CXG_EINVAL, "cxgServerWait: unknown ticket");
    const bool ok = S->done_cv.wait_for(
        g, std::chrono::duration<double>(timeout_s),
        [&] { return S->results[ticket].done; });
    if (!ok) return fail(CXG_ETIMEOUT, "cxgServerWait: not done yet");
    const SrvResult r = S->results[ticket];
    S->results.erase(ticket);
    if (lnL) *lnL = r.lnL;
    if (latency_ms) *latency_ms = r.latency_ms;
    if (r.rc) return fail(r.rc, "request failed: " + r.err);
    return 0;
}

extern "C" int cxgServerAddDataset(cxgServer *S, unsigned long long id, unsigned ntaxa,
                                   unsigned npat, const uint8_t *masks,
                                   const uint32_t *pattern_freqs) {
    if (S == nullptr || masks == nullptr || pattern_freqs == nullptr || id == 0)
        return fail(CXG_EINVAL, "cxgServerAddDataset: NULL or zero id");
    if (ntaxa < 3 || npat == 0) return fail(CXG_EINVAL, "cxgServerAddDataset: bad shape");
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (S->datasets.count(id)) return fail(CXG_EINVAL, "cxgServerAddDataset: id in use");
    }
    auto ds = std::make_unique<SrvDataset>();
    ds->hmasks.assign(masks, masks + (size_t)ntaxa * npat);
    ds->hfreqs.assign(pattern_freqs, pattern_freqs + npat);
    // Uploaded on the preparation stream and waited for here, so requests
    // that name the dataset may follow at once.
    int rc = upload_dataset(ntaxa, npat, masks, pattern_freqs, *ds, S->s_prep);
    if (rc == 0) {
        const cudaError_t e = cudaStreamSynchronize(S->s_prep);
        if (e != cudaSuccess) rc = cuda_fail(e, "cxgServerAddDataset");
    }
    if (rc) {
        if (ds->mem) dev_free(ds->mem);
        return rc;
    }
    std::lock_guard<std::mutex> g(S->mu);
    S->bytes_in_use += ds->bytes;
    S->bytes_peak = std::max(S->bytes_peak, S->bytes_in_use);
    S->datasets[id] = ds.release();
    return 0;
}

extern "C" int cxgServerAddDatasetRaw(cxgServer *S, unsigned long long id, unsigned ntaxa,
                                      unsigned nsites, const uint8_t *rows,
                                      const uint8_t *canon, const uint8_t *val,
                                      uint8_t any_mask, unsigned *npat) {
    if (S == nullptr || rows == nullptr || canon == nullptr || val == nullptr ||
        npat == nullptr || id == 0)
        return fail(CXG_EINVAL, "cxgServerAddDatasetRaw: NULL or zero id");
    if (ntaxa < 3 || nsites == 0)
        return fail(CXG_EINVAL, "cxgServerAddDatasetRaw: bad shape");
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (S->datasets.count(id)) return fail(CXG_EINVAL, "cxgServerAddDatasetRaw: id in use");
    }
    // The dataset keeps masks with row stride pad(nsites) >= pad(npat)
    // (pad patterns are "any"), weights and the leaf table; the raw rows
    // and the compaction scratch are freed afterwards.
    const unsigned N = ntaxa;
    const size_t stride = pad_patterns(nsites);
    auto ds = std::make_unique<SrvDataset>();
    ds->bytes = al256((size_t)N * stride) + al256((size_t)nsites * 4) +
                al256((size_t)N * sizeof(void *));
    ds->ntaxa = N;
    ds->stride = stride;
    cudaStream_t s = S->s_prep;
    const size_t work = compact_work_bytes(N, nsites);
    const size_t in_bytes = (size_t)N * nsites;
    char *tmp = nullptr;
    int rc = 0;
    cudaError_t e = dev_malloc_async((void **)&ds->mem, ds->bytes, s);
    if (e == cudaSuccess)
        e = dev_malloc_async((void **)&tmp, al256(in_bytes) + 1024 + 256 + work, s);
    if (e != cudaSuccess) {
        if (ds->mem) dev_free_async(ds->mem, s);
        cudaStreamSynchronize(s);
        return cuda_fail(e, "cxgServerAddDatasetRaw: device memory");
    }
    ds->masks = (uint8_t *)ds->mem;
    ds->weights = (uint32_t *)(ds->mem + al256((size_t)N * stride));
    ds->leaves = (const uint8_t **)(ds->mem + al256((size_t)N * stride) +
                                    al256((size_t)nsites * 4));
    uint8_t *d_rows = (uint8_t *)tmp;
    uint8_t *d_tab = (uint8_t *)tmp + al256(in_bytes);       // canon | val
    uint32_t *d_np = (uint32_t *)(d_tab + 512 + 256);
    void *d_work = tmp + al256(in_bytes) + 1024 + 256;
    uint8_t tabs[512];
    memcpy(tabs, canon, 256);
    memcpy(tabs + 256, val, 256);
    std::vector<const uint8_t *> hl(N);
    for (unsigned t = 0; t < N; ++t) hl[t] = ds->masks + (size_t)t * stride;
    uint32_t np = 0;
    if ((e = cudaMemcpyAsync(d_rows, rows, in_bytes, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(d_tab, tabs, 512, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(ds->leaves, hl.data(), N * sizeof(void *),
                             cudaMemcpyHostToDevice, s)))
        rc = cuda_fail(e, "cxgServerAddDatasetRaw: upload");
    if (rc == 0)
        rc = compact_device(d_rows, N, nsites, nullptr, canon, d_tab, d_tab + 256, any_mask,
                            nullptr, 0, ds->masks, (unsigned)stride, ds->weights, d_np,
                            d_work, work, s);
    if (rc == 0 && ((e = cudaMemcpyAsync(&np, d_np, 4, cudaMemcpyDeviceToHost, s)) ||
                    (e = cudaStreamSynchronize(s))))
        rc = cuda_fail(e, "cxgServerAddDatasetRaw: pattern count");
    if (rc == 0) {
        // Host copies for MC3 sessions built on this dataset.
        ds->npat = np;
        ds->hmasks.resize((size_t)N * np);
        ds->hfreqs.resize(np);
        if ((e = cudaMemcpy2DAsync(ds->hmasks.data(), np, ds->masks, stride, np, N,
                                   cudaMemcpyDeviceToHost, s)) ||
            (e = cudaMemcpyAsync(ds->hfreqs.data(), ds->weights, (size_t)np * 4,
                                 cudaMemcpyDeviceToHost, s)) ||
            (e = cudaStreamSynchronize(s)))
            rc = cuda_fail(e, "cxgServerAddDatasetRaw: host copy");
    }
    dev_free_async(tmp, s);
    if (rc) {
        dev_free_async(ds->mem, s);
        cudaStreamSynchronize(s);
        return rc;
    }
    *npat = np;
    std::lock_guard<std::mutex> g(S->mu);
    S->bytes_in_use += ds->bytes;
    S->bytes_peak = std::max(S->bytes_peak, S->bytes_in_use);
    S->datasets[id] = ds.release();
    return 0;
}

extern "C" int cxgServerDropDataset(cxgServer *S, unsigned long long id) {
    if (S == nullptr) return fail(CXG_EINVAL, "cxgServerDropDataset: NULL");
    SrvDataset *gone = nullptr;
    {
        std::lock_guard<std::mutex> g(S->mu);
        auto it = S->datasets.find(id);
        if (it == S->datasets.end())
            return fail(CXG_EINVAL, "cxgServerDropDataset: unknown dataset");
        SrvDataset *ds = it->second;
        S->datasets.erase(it);
        ds->dropped = true;
        if (ds->refs == 0) {
            S->bytes_in_use -= ds->bytes;
            gone = ds;
        }
    }
    if (gone) {
        dev_free(gone->mem);
        delete gone;
    }
    return 0;
}

extern "C" int cxgServerStats(cxgServer *S, cxgServerStatsT *st) {
    if (S == nullptr || st == nullptr) return fail(CXG_EINVAL, "cxgServerStats: NULL");
    std::lock_guard<std::mutex> g(S->mu);
    memset(st, 0, sizeof(*st));
    st->completed = S->completed;
    st->batches = S->batches;
    st->max_batch = S->max_batch;
    st->deferrals = S->deferrals;
    st->bytes_peak = S->bytes_peak;
    st->bytes_budget = S->budget;
    st->updates = S->updates_done;
    std::vector<double> l = S->latencies;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) {
            size_t i = (size_t)ceil(q * l.size()) - 1;
            if (i >= l.size()) i = l.size() - 1;
            return l[i];
        };
        st->p50_ms = pct(0.50);
        st->p99_ms = pct(0.99);
        st->max_ms = l.back();
        st->wall_s = std::chrono::duration<double>(S->t_last - S->t_first).count();
    }
    return 0;
}

extern "C" int cxgServerResetStats(cxgServer *S) {
    if (S == nullptr) return fail(CXG_EINVAL, "cxgServerResetStats: NULL");
    std::lock_guard<std::mutex> g(S->mu);
    S->latencies.clear();
    S->completed = S->batches = S->max_batch = S->deferrals = 0;
    S->updates_done = 0.0;
    S->any_done = false;
    return 0;
}

extern "C" int cxgServerDestroy(cxgServer *S) {
    if (S == nullptr) return 0;
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (auto &w : S->mc3_workers)
        if (w.joinable()) w.join();
    for (auto &kv : S->sessions) cxgMc3Destroy(kv.second.mc3);
    cudaStreamSynchronize(S->s_prep);
    for (auto &kv : S->datasets) {
        dev_free(kv.second->mem);
        delete kv.second;
    }
    for (auto &st : S->s_walk) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    S->stage.release();
    cudaStreamDestroy(S->s_prep);
    host_free(S->pinned);
    delete S;
    return 0;
}
