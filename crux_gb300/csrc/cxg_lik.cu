// Host side of the drop-in boundary: CL registry, plan translation and the
// extern "C" entry points of include/cxlik_gpu.h.
//
// The reference keeps each CL in host memory (Lik.pyx:60-107) and
// CxLikExecute reads/writes it there.  Here every host CxtLikCL is an
// identity: the registry maps its cLMat pointer to device buffers, internal
// CLs are computed and kept on the device, and leaf CLs are uploaded once as
// uint8 state masks.  A call translates lik->steps into a list of node
// updates (a Compute step followed by its Merge steps up to ntrail == 0,
// CxLik.c:314-596), uploads it in one copy, and launches two kernels: the
// P-matrix builder and the plan walker.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "cxg_internal.h"

namespace cxg {

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t err, const char *what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(err);
    return err == cudaErrorMemoryAllocation ? CXG_ENOMEM : CXG_ECUDA;
}

// Every device and pinned-host allocation of the library goes through
// these.  For tests (cxgDebugFailAllocs), g_alloc_budget >= 0 is the
// number of allocations that may still succeed; once it is spent, every
// allocation fails as an out-of-memory would, without calling CUDA.
static std::atomic<long long> g_alloc_budget{-1};

static bool alloc_allowed() {
    long long b = g_alloc_budget.load();
    while (b >= 0) {
        if (b == 0) return false;
        if (g_alloc_budget.compare_exchange_weak(b, b - 1)) return true;
    }
    return true;
}

// Debug canaries (cxgDebugCanaries, or CXG_DEBUG_CANARY set in the
// environment): every device allocation gets kCanaryBytes more, filled
// with kCanaryByte, and is tracked until it is freed.  A write past the end
// of a buffer changes its canary; cxgDebugCheckCanaries and every
// synchronous free read the canaries back.  This stands in for a memory
// checker on GPUs where none may run.
constexpr size_t kCanaryBytes = 256;
constexpr unsigned char kCanaryByte = 0xA5;
static std::mutex g_canary_mu;
static std::unordered_map<void *, size_t> g_canary;  // live allocation -> size
static std::atomic<int> g_canary_on{-1};               // -1: not yet read
static std::atomic<unsigned long long> g_canary_bad{0};

static bool canary_on() {
    int v = g_canary_on.load();
    if (v < 0) {
        v = getenv("CXG_DEBUG_CANARY") != nullptr ? 1 : 0;
        int expect = -1;
        g_canary_on.compare_exchange_strong(expect, v);
        v = g_canary_on.load();
    }
    return v > 0;
}

static void canary_track(void *p, size_t n) {
    std::lock_guard<std::mutex> g(g_canary_mu);
    g_canary[p] = n;
}

// Read one allocation's canary back (the device is idle); true if intact.
static bool canary_intact(void *p, size_t n) {
    unsigned char buf[kCanaryBytes];
    if (cudaMemcpy(buf, static_cast<char *>(p) + n, kCanaryBytes, cudaMemcpyDeviceToHost) !=
        cudaSuccess)
        return false;
    for (size_t i = 0; i < kCanaryBytes; ++i)
        if (buf[i] != kCanaryByte) return false;
    return true;
}

cudaError_t dev_malloc(void **p, size_t n) {
    if (!alloc_allowed()) return cudaErrorMemoryAllocation;
    if (!canary_on()) return cudaMalloc(p, n);
    cudaError_t e = cudaMalloc(p, n + kCanaryBytes);
    if (e != cudaSuccess) return e;
    e = cudaMemset(static_cast<char *>(*p) + n, kCanaryByte, kCanaryBytes);
    if (e == cudaSuccess) canary_track(*p, n);
    return e;
}

cudaError_t dev_malloc_async(void **p, size_t n, cudaStream_t s) {
    if (!alloc_allowed()) return cudaErrorMemoryAllocation;
    if (!canary_on()) return cudaMallocAsync(p, n, s);
    cudaError_t e = cudaMallocAsync(p, n + kCanaryBytes, s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(static_cast<char *>(*p) + n, kCanaryByte, kCanaryBytes, s);
    if (e == cudaSuccess) canary_track(*p, n);
    return e;
}

// Frees of the library's device allocations.  A synchronous free checks
// the canary first (after the device is idle); a stream-ordered one only
// stops tracking the buffer.
std::mutex &capture_gate() {
    static std::mutex m;
    return m;
}

cudaError_t host_free(void *p) {
    if (p == nullptr) return cudaSuccess;
    std::lock_guard<std::mutex> g(capture_gate());
    return cudaFreeHost(p);
}

cudaError_t device_sync() {
    std::lock_guard<std::mutex> g(capture_gate());
    return cudaDeviceSynchronize();
}

cudaError_t dev_free(void *p) {
    if (p == nullptr) return cudaSuccess;
    std::lock_guard<std::mutex> gate(capture_gate());
    if (canary_on()) {
        size_t n = 0;
        bool tracked = false;
        {
            std::lock_guard<std::mutex> g(g_canary_mu);
            auto it = g_canary.find(p);
            if (it != g_canary.end()) {
                n = it->second;
                tracked = true;
                g_canary.erase(it);
            }
        }
        if (tracked && cudaDeviceSynchronize() == cudaSuccess && !canary_intact(p, n))
            g_canary_bad.fetch_add(1);
    }
    return cudaFree(p);
}

cudaError_t dev_free_async(void *p, cudaStream_t s) {
    if (p == nullptr) return cudaSuccess;
    if (canary_on()) {
        std::lock_guard<std::mutex> g(g_canary_mu);
        g_canary.erase(p);
    }
    return cudaFreeAsync(p, s);
}

cudaError_t host_alloc(void **p, size_t n) {
    if (!alloc_allowed()) return cudaErrorMemoryAllocation;
    return cudaHostAlloc(p, n, cudaHostAllocDefault);
}


enum { CL_INTERNAL = 0, CL_LEAF = 1 };

struct DevCL {
    int kind = CL_INTERNAL;
    int precision = -1;   // precision of the data last written (internal)
    unsigned npat = 0, ppad = 0, kcap = 0;
    void *data = nullptr;
    void *scaler = nullptr;
    bool computed = false;
    // Translation that made this buffer a parent (State::gen); a child of
    // a later op in the same translation is then "written in this plan".
    unsigned long long gen = 0;
};

// Grow-only device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t n) {
        if (n <= cap) return 0;
        if (p) dev_free(p);
        p = nullptr;
        cap = 0;
        size_t want = n < 4096 ? 4096 : n + n / 2;
        cudaError_t e = dev_malloc(&p, want);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scratch)");
        cap = want;
        return 0;
    }
};

// Grow-only pinned host buffer.
struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t n) {
        if (n <= cap) return 0;
        if (p) host_free(p);
        p = nullptr;
        cap = 0;
        size_t want = n < 4096 ? 4096 : n + n / 2;
        cudaError_t e = host_alloc(&p, want);
        if (e != cudaSuccess) return cuda_fail(e, "cudaHostAlloc(staging)");
        cap = want;
        return 0;
    }
};

// Pattern weights on the device, one buffer per (host pointer, length),
// re-uploaded when the host content's hash changes.  Buffers are never
// shared between keys, so plans of different Liks never see each other's
// weights.
// Device copy of one pattern-weight array, with the host values it was
// made from: a call whose array (same pointer and length) still holds them
// reuses it.  The compare is a memcmp, exact and vectorised.
struct FreqEntry {
    DevBuf dev;
    std::vector<unsigned> host;
    // Registered by cxgLikSetPatternWeights: the caller keeps the host values
    // unchanged while registered, so calls skip the compare.
    bool registered = false;
};

struct State {
    std::mutex mu;
    bool ready = false;
    cudaStream_t stream = nullptr;
    std::unordered_map<uintptr_t, DevCL> cls;
    size_t cl_bytes = 0;
    size_t last_h2d = 0, last_d2h = 0;  // bytes copied by the last execute
    DevBuf misc;         // CxLikQDecomp in/out
    HostBuf stage, out;  // program staging, CxLikQDecomp staging
    // Recorded after each program upload from `stage`: the next translation
    // waits on it before it rewrites the staging buffer, so no upload has
    // to be waited for on the launch path.
    cudaEvent_t stage_ev = nullptr;
    bool stage_pending = false;
    std::unordered_map<std::string, FreqEntry> freqs;
    unsigned long long gen = 0;  // translations so far
    // Changes to the CL registry (a buffer allocated, replaced, forgotten or
    // cleared): a kept translation is valid only for the count it saw.
    unsigned long long epoch = 0;
    // The scratch plan's last translation, by the key of plan_key().
    std::vector<uint64_t> last_key;
    bool last_valid = false;
};

static State &state() {
    static State *s = new State();  // never destroyed: outlives callers
    return *s;
}

static int ensure_ready(State &S) {
    if (S.ready) return 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    CXG_CUDA(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    S.ready = true;
    return 0;
}

static void free_cl(State &S, DevCL &c) {
    if (c.data) dev_free(c.data);
    if (c.scaler) dev_free(c.scaler);
    size_t elt = (c.kind == CL_LEAF) ? 1 : (c.precision == CXG_FP32 ? 4 : 8);
    if (c.kind == CL_LEAF)
        S.cl_bytes -= c.ppad;
    else
        S.cl_bytes -= (size_t)c.kcap * 4 * c.ppad * elt + (size_t)c.ppad * 8;
    c.data = c.scaler = nullptr;
}

// Internal CL buffer for a parent written at `prec` with `kact` comps.
static int parent_buffer(State &S, const CxtLikCL *cl, unsigned npat,
                         unsigned kact, int prec, DevCL **out) {
    if (cl == nullptr || cl->cLMat == nullptr)
        return fail(CXG_EINVAL, "step parent CL has no cLMat");
    uintptr_t key = (uintptr_t)cl->cLMat;
    auto it = S.cls.find(key);
    const unsigned ppad = pad_patterns(npat);
    if (it != S.cls.end()) {
        DevCL &c = it->second;
        if (c.kind == CL_INTERNAL && c.precision == prec && c.npat == npat &&
            c.kcap >= kact) {
            *out = &c;
            return 0;
        }
        free_cl(S, c);
        S.cls.erase(it);
        ++S.epoch;
    }
    DevCL c;
    c.kind = CL_INTERNAL;
    c.precision = prec;
    c.npat = npat;
    c.ppad = ppad;
    c.kcap = kact;
    const size_t elt = prec == CXG_FP32 ? 4 : 8;
    CXG_CUDA(dev_malloc(&c.data, (size_t)kact * 4 * ppad * elt));
    cudaError_t e = dev_malloc(&c.scaler, (size_t)ppad * 8);
    if (e != cudaSuccess) {
        dev_free(c.data);
        return cuda_fail(e, "cudaMalloc(scaler)");
    }
    S.cl_bytes += (size_t)kact * 4 * ppad * elt + (size_t)ppad * 8;
    auto ins = S.cls.emplace(key, c);
    ++S.epoch;
    *out = &ins.first->second;
    return 0;
}

// Upload leaf masks.  zero_any: a 0 mask (gap) means "any state", as
// Lik.pyx:1469-1470 encodes it; otherwise a 0 mask stays a zero row.
static int upload_leaf(State &S, const double *key, const uint8_t *masks,
                       unsigned n, bool zero_any) {
    auto it = S.cls.find((uintptr_t)key);
    if (it != S.cls.end()) {
        free_cl(S, it->second);
        S.cls.erase(it);
    }
    ++S.epoch;
    DevCL c;
    c.kind = CL_LEAF;
    c.npat = n;
    c.ppad = pad_patterns(n);
    c.computed = true;
    std::vector<uint8_t> h(c.ppad, 15);  // pad patterns: all states allowed
    for (unsigned i = 0; i < n; ++i)
        h[i] = (masks[i] & 15) ? (masks[i] & 15) : (zero_any ? 15 : 0);
    CXG_CUDA(dev_malloc(&c.data, c.ppad));
    cudaError_t e = cudaMemcpy(c.data, h.data(), c.ppad, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        dev_free(c.data);
        return cuda_fail(e, "cudaMemcpy(leaf masks)");
    }
    S.cl_bytes += c.ppad;
    S.cls.emplace((uintptr_t)key, c);
    return 0;
}

// Leaf child used by a plan: registered masks, or (drop-in path) the host
// rows of 4 doubles written by Lik.pyx:1466-1475.
static int leaf_child(State &S, const CxtLik *lik, const CxtLikCL *cl,
                      DevCL **out) {
    if (cl == nullptr || cl->cLMat == nullptr)
        return fail(CXG_EINVAL, "leaf child CL has no cLMat");
    uintptr_t key = (uintptr_t)cl->cLMat;
    auto it = S.cls.find(key);
    if (it == S.cls.end() || it->second.kind != CL_LEAF ||
        it->second.npat != lik->mschars) {
        std::vector<uint8_t> m(lik->mschars);
        for (unsigned c = 0; c < lik->mschars; ++c) {
            unsigned v = 0;
            for (unsigned j = 0; j < 4; ++j) {
                double x = cl->cLMat[c * 4 + j];
                if (x == 1.0)
                    v |= 1u << j;
                else if (x != 0.0)
                    return fail(CXG_EINVAL,
                                "leaf CL rows must hold 0/1 state indicators");
            }
            m[c] = (uint8_t)v;
        }
        // A row of zeros keeps mask 0, whose message is all zeros, as the
        // reference computes it.
        int rc = upload_leaf(S, cl->cLMat, m.data(), lik->mschars, false);
        if (rc) return rc;
        it = S.cls.find(key);
    }
    *out = &it->second;
    return 0;
}

// Internal child: computed by an earlier run at this precision, or by an
// earlier op of the plan being translated (translation `gen`).
static int internal_child(State &S, const CxtLik *lik, const CxtLikCL *cl,
                          unsigned kact, int prec, unsigned long long gen,
                          DevCL **out) {
    if (cl == nullptr || cl->cLMat == nullptr)
        return fail(CXG_EINVAL, "internal child CL has no cLMat");
    auto it = S.cls.find((uintptr_t)cl->cLMat);
    const bool earlier = it != S.cls.end() && it->second.gen == gen;
    if (it == S.cls.end() || it->second.kind != CL_INTERNAL ||
        !(it->second.computed || earlier) || it->second.precision != prec ||
        it->second.npat != lik->mschars || it->second.kcap < kact)
        return fail(CXG_EINVAL,
                    "plan reads a child CL that has not been computed on the "
                    "device at this precision");
    *out = &it->second;
    return 0;
}

// A translated plan: the device program of one lik->steps list at one
// precision, runnable any number of times.  CL buffers it references must
// outlive it.
struct Plan {
    int prec = CXG_FP64;
    unsigned npat = 0, ppad = 0, kact = 0, nops = 0, nchild = 0;
    DevBuf prog, partial, misc, ltab;
    HostBuf out;
    DevCL *root = nullptr;
    std::vector<DevCL *> parents;
    PmatArgs pa;
    PlanArgs a;
    double alg_bytes = 0.0;   // algorithmic bytes of one plan-walker launch
    double updates = 0.0;     // pattern-node updates of one run
    unsigned tile = kTile, tpp = 1, ppt = 1, nslot = 0, nleaf = 0;
    unsigned lanes = 1;       // op lanes of the walker (records per step)
    // Where the per-call values sit in the program (byte offsets): branch
    // lengths [stepsLen], cmult, rmult, model index [kact], cube and
    // eigenvalues [models], root weights pn [kact][4]; and what they are
    // read from (active components, their models).
    size_t o_elen = 0, o_cm = 0, o_rm = 0, o_mod = 0, o_cube = 0, o_eig = 0,
           o_dst = 0, o_pn = 0;
    std::vector<unsigned> act;
    std::vector<const CxtLikModel *> models;
    std::vector<int32_t> model_of;
};

// Launch shape of the plan walker: patterns per CTA, threads per pattern
// and the shared-memory budget of the CL stack (set by cxgTune).
// Device copy of lik's pattern weights, one per (host pointer, length),
// uploaded again whenever the host values differ from the kept copy.
static int pattern_weights(State &S, const CxtLik *lik, const void **out) {
    const unsigned npat = lik->mschars;
    const unsigned *fh = lik->charFreqs + lik->cbase;
    char key[64];
    snprintf(key, sizeof(key), "%p:%u", (const void *)fh, npat);
    FreqEntry &fe = S.freqs[key];
    if (fe.registered && fe.dev.p != nullptr && fe.host.size() == npat) {
        *out = fe.dev.p;
        return 0;
    }
    if (fe.dev.p == nullptr || fe.host.size() != npat ||
        memcmp(fe.host.data(), fh, (size_t)npat * 4) != 0) {
        int rc = fe.dev.ensure((size_t)npat * 4);
        if (rc) return rc;
        CXG_CUDA(cudaMemcpy(fe.dev.p, fh, (size_t)npat * 4, cudaMemcpyHostToDevice));
        fe.host.assign(fh, fh + npat);
    }
    *out = fe.dev.p;
    return 0;
}

// The per-call values of a translated plan, into program image h: every
// step's branch length (each step has one child, so child c is step c),
// the active components' cmult, rmult, model index and root weights, and
// each model's eigenvector cube and eigenvalues.
static void pack_values(const CxtLik *lik, const Plan &P, char *h) {
    double *el = reinterpret_cast<double *>(h + P.o_elen);
    for (unsigned s = 0; s < lik->stepsLen; ++s) el[s] = lik->steps[s].edgeLen;
    for (unsigned k = 0; k < P.kact; ++k) {
        const CxtLikComp &cp = lik->comps[P.act[k]];
        reinterpret_cast<double *>(h + P.o_cm)[k] = cp.cmult;
        reinterpret_cast<double *>(h + P.o_rm)[k] = cp.model->rmult;
        reinterpret_cast<int32_t *>(h + P.o_mod)[k] = P.model_of[k];
        for (unsigned i = 0; i < 4; ++i)
            reinterpret_cast<double *>(h + P.o_pn)[k * 4 + i] =
                cp.model->piDiagNorm[i] * cp.weightScaled;
    }
    for (size_t m = 0; m < P.models.size(); ++m) {
        memcpy(h + P.o_cube + m * 64 * 8, P.models[m]->qEigVecCube, 64 * 8);
        memcpy(h + P.o_eig + m * 4 * 8, P.models[m]->qEigVals, 4 * 8);
    }
}

static unsigned g_tile = kTile;
static unsigned g_tpp = 1;
static unsigned g_ppt = 1;
static unsigned g_lanes = 1;
static size_t g_smem_budget = 24 * 1024;

static int translate(State &S, CxtLik *lik, int prec, Plan &P,
                     bool use_slots = true, bool allow_lanes = false) {
    int rc;
    if (lik == nullptr) return fail(CXG_EINVAL, "lik is NULL");
    if (lik->dim != 4)
        return fail(CXG_EINVAL, "only 4-state (DNA) likelihoods run on the GPU");
    if (prec != CXG_FP64 && prec != CXG_FP32)
        return fail(CXG_EINVAL, "unknown precision");
    const unsigned npat = lik->mschars;
    if (npat == 0) return fail(CXG_EINVAL, "mschars is 0");
    const unsigned ppad = pad_patterns(npat);

    // Active components and the models they use.
    std::vector<unsigned> act;
    for (unsigned mc = 0; mc < lik->compsLen; ++mc)
        if (lik->comps[mc].weightScaled != 0.0) act.push_back(mc);
    const unsigned kact = (unsigned)act.size();
    if (kact == 0) return fail(CXG_EINVAL, "no component has non-zero weight");
    if (kact > kMaxComps)
        return fail(CXG_EINVAL, "more than 8 active mixture components");
    std::vector<const CxtLikModel *> models;
    std::vector<int32_t> model_of(kact);
    for (unsigned k = 0; k < kact; ++k) {
        const CxtLikModel *m = lik->comps[act[k]].model;
        int idx = -1;
        for (size_t i = 0; i < models.size(); ++i)
            if (models[i] == m) idx = (int)i;
        if (idx < 0) {
            idx = (int)models.size();
            models.push_back(m);
        }
        model_of[k] = idx;
    }

    // Group steps into node updates.
    struct HostOp {
        void *data, *scaler;
        uint32_t child0, nchild;
        int slot;
    };
    struct HostChild {
        const void *data, *scaler;
        uint32_t src, idx;
        int32_t tab;
    };
    std::vector<HostOp> ops;
    std::vector<HostChild> kids;
    std::vector<double> elen;
    std::vector<DevCL *> kid_cl;
    int32_t ntab = 0;
    P.parents.clear();
    const unsigned long long gen = ++S.gen;
    const CxtLikCL *cur_parent = nullptr;
    unsigned expect_trail = 0;
    const double s_el = prec == CXG_FP32 ? 4.0 : 8.0;
    const double e_el = prec == CXG_FP32 ? 4.0 : 8.0;
    double bytes = 0.0;
    for (unsigned s = 0; s < lik->stepsLen; ++s) {
        const CxtLikStep &st = lik->steps[s];
        if ((unsigned)st.variant > 3) return fail(CXG_EINVAL, "bad step variant");
        const bool compute = (st.variant == CxeLikStepComputeL ||
                              st.variant == CxeLikStepComputeI);
        const bool leaf = (st.variant == CxeLikStepComputeL ||
                           st.variant == CxeLikStepMergeL);
        if (compute) {
            if (cur_parent != nullptr)
                return fail(CXG_EINVAL, "Compute step before ntrail reached 0");
            DevCL *pc = nullptr;
            rc = parent_buffer(S, st.parentCL, npat, kact, prec, &pc);
            if (rc) return rc;
            HostOp op;
            op.data = pc->data;
            op.scaler = pc->scaler;
            op.child0 = (uint32_t)kids.size();
            op.nchild = 0;
            op.slot = -1;
            ops.push_back(op);
            P.parents.push_back(pc);
            pc->gen = gen;
            cur_parent = st.parentCL;
            bytes += 4.0 * kact * s_el + e_el;  // parent written
        } else {
            if (cur_parent == nullptr || st.parentCL != cur_parent ||
                st.ntrail + 1 != expect_trail)
                return fail(CXG_EINVAL, "Merge step does not continue its node");
        }
        DevCL *cc = nullptr;
        rc = leaf ? leaf_child(S, lik, st.childCL, &cc)
                  : internal_child(S, lik, st.childCL, kact, prec, gen,
                                   &cc);
        if (rc) return rc;
        if (cc->data == P.parents.back()->data)
            return fail(CXG_EINVAL, "step reads its own parent");
        HostChild ch;
        ch.data = cc->data;
        ch.scaler = leaf ? nullptr : cc->scaler;
        ch.src = leaf ? SRC_LEAF : SRC_GLOBAL;
        ch.idx = 0;
        // Leaf children: an FP64 table index, or (FP32) >= 0 for the table
        // in the record.
        ch.tab = leaf ? (prec == CXG_FP64 ? ntab++ : 0) : -1;
        kids.push_back(ch);
        kid_cl.push_back(cc);
        elen.push_back(st.edgeLen);
        bytes += leaf ? 1.0 : 4.0 * kact * s_el + e_el;  // child read
        if (ops.back().nchild + 1u > kMaxChildren)
            return fail(CXG_EINVAL, "node degree above 17");
        ops.back().nchild++;
        expect_trail = st.ntrail;
        if (st.ntrail == 0) cur_parent = nullptr;
    }
    if (cur_parent != nullptr) return fail(CXG_EINVAL, "plan ends mid-node");

    // Root CL.
    if (lik->rootCLC == nullptr || lik->rootCLC->cLMat == nullptr)
        return fail(CXG_EINVAL, "rootCLC has no cLMat");
    {
        auto it = S.cls.find((uintptr_t)lik->rootCLC->cLMat);
        if (it == S.cls.end() || it->second.kind != CL_INTERNAL ||
            it->second.precision != prec || it->second.kcap < kact)
            return fail(CXG_EINVAL, "root CL has not been computed");
        P.root = &it->second;
        bool in_plan = false;
        for (DevCL *p : P.parents) in_plan |= (p == P.root);
        if (!in_plan && !P.root->computed)
            return fail(CXG_EINVAL, "root CL has not been computed");
    }
    bytes += 4.0 * kact * s_el + e_el + 4.0 + 8.0;  // root read, freq, site

    // Leaves: staged once per tile (each distinct leaf one row, named by
    // kids[c].idx) when they fit kLeafStageBytes, else each op's mask
    // arrays (kids[c].data) travel with its record (lmax rows per stage).
    const unsigned tile = g_tile;
    std::vector<const uint8_t *> leaf_ptrs;
    unsigned lmax = 0;
    {
        std::unordered_map<DevCL *, uint32_t> leaf_idx;
        for (size_t c = 0; c < kids.size(); ++c) {
            if (kids[c].src != SRC_LEAF) continue;
            auto it = leaf_idx.find(kid_cl[c]);
            if (it == leaf_idx.end()) {
                it = leaf_idx.emplace(kid_cl[c], (uint32_t)leaf_ptrs.size()).first;
                leaf_ptrs.push_back(static_cast<const uint8_t *>(kid_cl[c]->data));
            }
            kids[c].idx = it->second;
        }
        for (const HostOp &op : ops) {
            unsigned n = 0;
            for (uint32_t c = op.child0; c < op.child0 + op.nchild; ++c)
                n += kids[c].src == SRC_LEAF;
            if (n > lmax) lmax = n;
        }
    }
    const unsigned nleaf = (unsigned)leaf_ptrs.size();
    const bool stage_leaves = (size_t)nleaf * tile <= kLeafStageBytes;
    const unsigned s_lmax = stage_leaves ? 0 : lmax;
    const unsigned s_nleaf = stage_leaves ? nleaf : 0;

    // Shared-memory stack: a parent keeps a slot until its one consumer (a
    // later op of this run) reads it; with no free slot the oldest holder
    // loses its slot and its consumer reads the HBM copy instead.
    // Record stride: the largest op's header, children and child areas.
    size_t rstride = 16;
    std::vector<size_t> rec_bytes(ops.size());  // each op's record, 16-byte units
    for (size_t o = 0; o < ops.size(); ++o) {
        const HostOp &op = ops[o];
        size_t b = sizeof(RecHead) + op.nchild * sizeof(RecChild);
        for (uint32_t c = op.child0; c < op.child0 + op.nchild; ++c)
            b += child_area_bytes(prec, kact, kids[c].src == SRC_LEAF);
        b = (b + 15) & ~(size_t)15;
        rec_bytes[o] = b;
        if (b > rstride) rstride = b;
    }
    const bool root_last = !ops.empty() && P.parents.back() == P.root;
    const unsigned tpp = tuned_tpp(prec, kact, tile);
    const unsigned ppt = tuned_ppt(prec, kact, tile, tpp);
    // Op lanes: two mutually independent ops per step (single plans of the
    // FP32 form with staged leaves, when tuned so).
    const unsigned lanes =
        (allow_lanes && g_lanes == 2 && stage_leaves && ops.size() >= 2 &&
         lanes_shape_ok(prec, kact, tpp, ppt) && tile * 2 <= kLaneThreads)
            ? 2u : 1u;
    // order[r]: the op in record position r, or -1 for an empty lane.  With
    // lanes, each op goes to the earliest step after those of the ops that
    // produce its children (ops in post-order, steps filled in that order),
    // and the root takes the last step alone, in lane 0.
    std::vector<int> order;
    if (lanes == 1) {
        order.resize(ops.size());
        for (size_t o = 0; o < ops.size(); ++o) order[o] = (int)o;
    } else {
        std::unordered_map<DevCL *, int> prod;
        for (size_t o = 0; o < ops.size(); ++o) prod[P.parents[o]] = (int)o;
        std::vector<int> step_of(ops.size(), 0);
        std::vector<unsigned> fill;
        for (size_t o = 0; o < ops.size(); ++o) {
            size_t lo = 0;
            for (uint32_t c = ops[o].child0; c < ops[o].child0 + ops[o].nchild; ++c) {
                if (kids[c].src == SRC_LEAF) continue;
                auto it = prod.find(kid_cl[c]);
                if (it != prod.end() && it->second < (int)o)
                    lo = std::max(lo, (size_t)step_of[it->second] + 1);
            }
            const bool alone = root_last && o + 1 == ops.size();
            if (alone) lo = std::max(lo, fill.size());
            size_t st = lo;
            while (st < fill.size() && fill[st] >= lanes) ++st;
            if (st >= fill.size()) fill.resize(st + 1, 0);
            step_of[o] = (int)st;
            fill[st] += alone ? lanes : 1u;
        }
        order.assign(fill.size() * lanes, -1);
        std::vector<unsigned> n_in(fill.size(), 0);
        for (size_t o = 0; o < ops.size(); ++o) {
            const size_t st = (size_t)step_of[o];
            order[st * lanes + n_in[st]++] = (int)o;
        }
    }
    // A stage of the lane walker holds two records: half the stages keep
    // as many records in flight.
    const unsigned ring = lanes == 2 ? kRing / 2 : kRing;
    const unsigned sbytes = (unsigned)rstride * lanes;  // one ring stage
    const size_t base_bytes = plan_smem_bytes(prec, kact, tile, 0, ring,
                                              sbytes, s_lmax, s_nleaf);
    const size_t slot_bytes =
        plan_smem_bytes(prec, kact, tile, 1, ring, sbytes, s_lmax, s_nleaf) -
        base_bytes;
    unsigned cap = 0;
    if (g_smem_budget > base_bytes)
        cap = (unsigned)((g_smem_budget - base_bytes) / slot_bytes);
    if (cap > kMaxSlots) cap = kMaxSlots;
    if (!use_slots) cap = 0;
    unsigned used = 0;
    {
        // Step by step: every child the step's ops read is taken first, so a
        // slot they free can hold a result of the same step (results are
        // stored after the step's release barrier); a slot assigned in this
        // step is never taken again in it, since both lanes would store it.
        std::vector<int> owner(cap, -1);                 // op holding slot
        std::vector<size_t> owner_step(cap, 0);
        std::unordered_map<DevCL *, int> made;           // parent -> op
        const size_t nsteps = order.size() / lanes;
        for (size_t st = 0; st < nsteps; ++st) {
            for (unsigned l = 0; l < lanes; ++l) {
                const int o = order[st * lanes + l];
                if (o < 0) continue;
                for (uint32_t c = ops[o].child0; c < ops[o].child0 + ops[o].nchild; ++c) {
                    if (kids[c].src == SRC_LEAF) continue;
                    auto it = made.find(kid_cl[c]);
                    if (it == made.end()) continue;      // from an earlier run
                    const int prod = it->second;
                    const int sl = ops[prod].slot;
                    if (sl >= 0 && owner[sl] == prod) {
                        kids[c].src = SRC_SLOT;
                        kids[c].idx = (uint32_t)sl;
                        owner[sl] = -1;
                    }
                    made.erase(it);
                }
            }
            for (unsigned l = 0; l < lanes; ++l) {
                const int o = order[st * lanes + l];
                if (o < 0) continue;
                if ((size_t)o + 1 == ops.size() || cap == 0) continue;  // root: no slot
                int sl = -1;
                for (unsigned k = 0; k < cap && sl < 0; ++k)
                    if (owner[k] < 0) sl = (int)k;
                if (sl < 0) {
                    int oldest = -1;
                    for (unsigned k = 0; k < cap; ++k)
                        if (owner_step[k] != st &&
                            (oldest < 0 || owner[k] < owner[oldest]))
                            oldest = (int)k;
                    sl = oldest;
                }
                if (sl < 0) continue;  // every slot taken in this step
                owner[sl] = o;
                owner_step[sl] = st;
                ops[o].slot = sl;
                made[P.parents[o]] = o;
                if ((unsigned)sl + 1 > used) used = (unsigned)sl + 1;
            }
        }
    }
    const unsigned nslot = used;

    // Pattern weights, one device copy per (host pointer, length).
    const void *dfreqs = nullptr;
    rc = pattern_weights(S, lik, &dfreqs);
    if (rc) return rc;

    // Pack the program into pinned staging, one copy:
    //   records [nops][rstride] | elen | cmult | rmult | model | cube | eig |
    //   dst | pn
    const unsigned nchild = (unsigned)kids.size();
    const unsigned nmod = (unsigned)models.size();
    auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
    const size_t nrec = order.empty() ? 1 : order.size();
    size_t o_rec = 0;
    size_t o_elen = al(o_rec + nrec * rstride);
    size_t o_cm = al(o_elen + elen.size() * 8);
    size_t o_rm = al(o_cm + kact * 8);
    size_t o_mod = al(o_rm + kact * 8);
    size_t o_cube = al(o_mod + kact * 4);
    size_t o_eig = al(o_cube + nmod * 64 * 8);
    size_t o_dst = al(o_eig + nmod * 4 * 8);
    size_t o_tab = al(o_dst + (size_t)nchild * 8);
    size_t o_pn = al(o_tab + (size_t)nchild * 4);
    size_t o_lrow = al(o_pn + kact * 4 * 8);
    size_t o_leaf = al(o_lrow + (nrec * (s_lmax ? s_lmax : 1)) * sizeof(void *));
    size_t total = al(o_leaf + (s_nleaf ? s_nleaf : 1) * sizeof(void *));
    if (S.stage_pending) {
        CXG_CUDA(cudaEventSynchronize(S.stage_ev));
        S.stage_pending = false;
    }
    rc = S.stage.ensure(total);
    if (rc) return rc;
    rc = P.prog.ensure(total);
    if (rc) return rc;
    char *h = static_cast<char *>(S.stage.p);
    // Record bytes are not zeroed: every header and child descriptor is
    // written whole below, the child areas by the P kernel, and no kernel
    // reads a record past its own bytes.
    uint64_t *dsts = (uint64_t *)(h + o_dst);
    for (size_t pos = 0; pos < order.size(); ++pos) {
        char *r = h + o_rec + pos * rstride;
        RecHead hd;
        memset(&hd, 0, sizeof(hd));
        if (order[pos] < 0) {  // an empty lane: no children, no result
            hd.slot = -1;
            hd.flags = REC_NO_HBM;
            memcpy(r, &hd, sizeof(hd));
            continue;
        }
        const size_t o = (size_t)order[pos];
        if (lanes == 1 && pos + ring < order.size())
            hd.next_bytes = (uint32_t)rec_bytes[order[pos + ring]];
        hd.data = ops[o].data;
        hd.scaler = ops[o].scaler;
        hd.nchild = ops[o].nchild;
        hd.slot = ops[o].slot;
        if (prec == CXG_FP32 && lanes == 1 && ops[o].nchild == 2) {
            const HostChild &k0 = kids[ops[o].child0], &k1 = kids[ops[o].child0 + 1];
            hd.flags |= op_kind_flags(k0.src, k0.data, k1.src, k1.data,
                                      pos > 0 ? ops[order[pos - 1]].data : nullptr);
        }
        memcpy(r, &hd, sizeof(hd));
        size_t area = sizeof(RecHead) + ops[o].nchild * sizeof(RecChild);
        for (uint32_t ci = 0; ci < ops[o].nchild; ++ci) {
            const HostChild &k = kids[ops[o].child0 + ci];
            const size_t ab = child_area_bytes(prec, kact, k.src == SRC_LEAF);
            if (area + ab > rstride)
                return fail(CXG_EINVAL, "internal: child area outside its record");
            RecChild rc_;
            memset(&rc_, 0, sizeof(rc_));
            rc_.data = k.data;
            rc_.scaler = k.scaler;
            rc_.src = k.src;
            rc_.idx = k.idx;
            rc_.tab = k.tab < 0 ? 0u : (uint32_t)k.tab;
            rc_.off = (uint32_t)area;
            memcpy(r + sizeof(RecHead) + ci * sizeof(RecChild), &rc_, sizeof(rc_));
            // Byte offset from the start of the records (pa.rec).
            dsts[ops[o].child0 + ci] = pos * rstride + area;
            area += ab;
        }
    }
    for (unsigned c = 0; c < nchild; ++c) ((int32_t *)(h + o_tab))[c] = kids[c].tab;
    P.kact = kact;
    P.o_elen = o_elen;
    P.o_cm = o_cm;
    P.o_rm = o_rm;
    P.o_mod = o_mod;
    P.o_cube = o_cube;
    P.o_eig = o_eig;
    P.o_dst = o_dst;
    P.o_pn = o_pn;
    P.act = act;
    P.models = models;
    P.model_of = model_of;
    pack_values(lik, P, h);
    {
        // Streamed: leaf rows of each op in child order, null-terminated.
        // Staged: the leaf table.
        const void **lr = reinterpret_cast<const void **>(h + o_lrow);
        memset(lr, 0, nrec * (s_lmax ? s_lmax : 1) * sizeof(void *));
        for (size_t o = 0; o < ops.size() && s_lmax; ++o) {
            unsigned j = 0;
            for (uint32_t c = ops[o].child0; c < ops[o].child0 + ops[o].nchild; ++c)
                if (kids[c].src == SRC_LEAF) lr[o * s_lmax + j++] = kids[c].data;
        }
        if (s_nleaf) memcpy(h + o_leaf, leaf_ptrs.data(), s_nleaf * sizeof(void *));
    }
    char *d = static_cast<char *>(P.prog.p);
    CXG_CUDA(cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, S.stream));
    S.last_h2d = total;
    if (S.stage_ev == nullptr)
        CXG_CUDA(cudaEventCreateWithFlags(&S.stage_ev, cudaEventDisableTiming));
    CXG_CUDA(cudaEventRecord(S.stage_ev, S.stream));
    S.stage_pending = true;

    PmatArgs &pa = P.pa;
    pa.nchild = nchild;
    pa.kact = kact;
    pa.precision = prec;
    pa.edge_len = (const double *)(d + o_elen);
    pa.cmult = (const double *)(d + o_cm);
    pa.rmult = (const double *)(d + o_rm);
    pa.model = (const int32_t *)(d + o_mod);
    pa.cube = (const double *)(d + o_cube);
    pa.eig = (const double *)(d + o_eig);
    pa.dst = (const uint64_t *)(d + o_dst);
    pa.tab = (const int32_t *)(d + o_tab);
    pa.wnorm = lik->wNorm;
    pa.wnorm_dev = nullptr;
    pa.rec = (unsigned char *)(d + o_rec);
    rc = P.ltab.ensure((size_t)(ntab ? ntab : 1) * 16 * kact * 4 * 8);
    if (rc) return rc;
    pa.ltab = (double *)P.ltab.p;

    const unsigned nb = plan_blocks(ppad, tile);
    rc = P.partial.ensure((size_t)nb * 16);
    if (rc) return rc;
    // misc: ticket (4) | ninf (4) | err (4) | pad (4) | total (16) | site
    rc = P.misc.ensure(32 + (size_t)ppad * 8);
    if (rc) return rc;
    rc = P.out.ensure(32);
    if (rc) return rc;
    char *mp = static_cast<char *>(P.misc.p);
    PlanArgs &a = P.a;
    a.rec = (const unsigned char *)(d + o_rec);
    a.lrows = (const uint8_t *const *)(d + o_lrow);
    a.lmax = s_lmax;
    a.leaves = (const uint8_t *const *)(d + o_leaf);
    a.nleaf = s_nleaf;
    a.rstride = (uint32_t)rstride;
    a.ring = ring;
    a.nslot = nslot;
    a.tile = tile;
    a.tpp = tpp;
    a.ppt = ppt;
    a.root_last = root_last ? 1u : 0u;
    a.nops = (uint32_t)order.size();  // records, empty lanes included
    a.kact = kact;
    a.npat = npat;
    a.ppad = ppad;
    a.pn = (const double *)(d + o_pn);
    a.root = P.root->data;
    a.rootsc = P.root->scaler;
    a.freqs = (const uint32_t *)dfreqs;
    a.site = nullptr;
    a.partial = (double *)P.partial.p;
    a.ticket = (unsigned *)mp;
    a.ninf = (uint32_t *)(mp + 4);
    a.err = (uint32_t *)(mp + 8);
    a.total = (double *)(mp + 16);
    a.ltab = (const double *)P.ltab.p;
    a.ntiles = nb;
    a.no_root = 0;
    P.prec = prec;
    P.npat = npat;
    P.ppad = ppad;
    P.kact = kact;
    P.nops = (unsigned)ops.size();
    P.nchild = nchild;
    P.alg_bytes = bytes * npat;
    P.updates = (double)ops.size() * npat;
    P.tile = tile;
    P.tpp = a.tpp;
    P.ppt = a.ppt;
    P.lanes = lanes;
    P.nslot = nslot;
    P.nleaf = nleaf;
    return 0;
}

// Enqueue one run (P matrices, plan walk, result copy) on the stream;
// optional events bracket the plan-walker launch.
// `pdl`: the walker is a programmatic dependent of the P kernel (not with
// timing events, whose walker span must be the walker alone).
static int enqueue(State &S, Plan &P, bool want_site,
                   cudaEvent_t e0 = nullptr, cudaEvent_t e1 = nullptr,
                   bool pdl = false) {
    char *mp = static_cast<char *>(P.misc.p);
    P.a.site = want_site ? (double *)(mp + 32) : nullptr;
    // The P kernel clears the walker's 32 result bytes; a plan with no P
    // matrices clears them with a memset.
    const bool pmat = P.pa.nchild * P.pa.kact > 0;
    P.pa.zero = pmat ? reinterpret_cast<uint64_t *>(mp) : nullptr;
    if (!pmat) CXG_CUDA(cudaMemsetAsync(mp, 0, 32, S.stream));
    CXG_CUDA(launch_pmat(P.pa, S.stream));
    if (e0) CXG_CUDA(cudaEventRecord(e0, S.stream));
    CXG_CUDA(launch_plan(P.prec, P.a, S.stream, P.lanes,
                         pdl && e0 == nullptr && P.pa.nchild > 0));
    if (e1) CXG_CUDA(cudaEventRecord(e1, S.stream));
    CXG_CUDA(cudaMemcpyAsync(P.out.p, mp, 32, cudaMemcpyDeviceToHost, S.stream));
    return 0;
}

static int finish(State &S, Plan &P, double *lnL, double *site) {
    if (site)
        CXG_CUDA(cudaMemcpyAsync(site, static_cast<char *>(P.misc.p) + 32,
                                 (size_t)P.npat * 8, cudaMemcpyDeviceToHost,
                                 S.stream));
    CXG_CUDA(cudaStreamSynchronize(S.stream));
    const char *o = static_cast<const char *>(P.out.p);
    uint32_t ninf, err;
    double tot[2];
    memcpy(&ninf, o + 4, 4);
    memcpy(&err, o + 8, 4);
    memcpy(tot, o + 16, 16);
    // A walk that gave up leaves its parents partly written: a later plan
    // may not read them as children until they are recomputed.
    for (DevCL *p : P.parents) p->computed = (err == 0);
    if (err)
        return fail(CXG_ETIMEOUT,
                    "plan walker: an op-record copy did not complete in time");
    if (lnL) *lnL = ninf ? -INFINITY : tot[0] + tot[1];
    return 0;
}

static void free_plan(Plan &P) {
    if (P.prog.p) dev_free(P.prog.p);
    if (P.ltab.p) dev_free(P.ltab.p);
    if (P.partial.p) dev_free(P.partial.p);
    if (P.misc.p) dev_free(P.misc.p);
    if (P.out.p) host_free(P.out.p);
    P.prog = DevBuf();
    P.ltab = DevBuf();
    P.partial = DevBuf();
    P.misc = DevBuf();
    P.out = HostBuf();
}

static Plan &scratch_plan() {
    static Plan *p = new Plan();
    return *p;
}

// Everything a translation depends on apart from the per-call values: the
// launch shape and precision, the registry state, the Lik's sizes, which
// components are active with which models, the root, and every step's
// variant, ntrail and CLs (struct and buffer).  Branch lengths, model
// parameters, wNorm and the pattern weights are values.
static void plan_key(const State &S, const CxtLik *lik, int prec,
                     std::vector<uint64_t> &k) {
    k.clear();
    k.reserve(16 + lik->compsLen + 5 * (size_t)lik->stepsLen);
    k.push_back((uint64_t)prec);
    k.push_back(g_tile);
    k.push_back(g_tpp);
    k.push_back(g_ppt);
    k.push_back(g_smem_budget);
    k.push_back(g_lanes);
    k.push_back(S.epoch);
    k.push_back((uintptr_t)lik);
    k.push_back(lik->dim);
    k.push_back(lik->mschars);
    k.push_back(lik->cbase);
    k.push_back((uintptr_t)lik->rootCLC);
    k.push_back(lik->rootCLC ? (uintptr_t)lik->rootCLC->cLMat : 0);
    k.push_back(lik->compsLen);
    for (unsigned c = 0; c < lik->compsLen; ++c)
        k.push_back(lik->comps[c].weightScaled != 0.0 ? (uintptr_t)lik->comps[c].model : 0);
    k.push_back(lik->stepsLen);
    for (unsigned i = 0; i < lik->stepsLen; ++i) {
        const CxtLikStep &st = lik->steps[i];
        k.push_back(((uint64_t)(uint32_t)st.variant << 32) | st.ntrail);
        k.push_back((uintptr_t)st.parentCL);
        k.push_back(st.parentCL ? (uintptr_t)st.parentCL->cLMat : 0);
        k.push_back((uintptr_t)st.childCL);
        k.push_back(st.childCL ? (uintptr_t)st.childCL->cLMat : 0);
    }
}

// Reuse the scratch plan's translation for a call with the same key:
// write the values into the staging image and upload only them (the
// records, child descriptors and tables on the device are unchanged).
static int refresh_values(State &S, CxtLik *lik, Plan &P) {
    const void *dfreqs = nullptr;
    int rc = pattern_weights(S, lik, &dfreqs);
    if (rc) return rc;
    if (S.stage_pending) {
        CXG_CUDA(cudaEventSynchronize(S.stage_ev));
        S.stage_pending = false;
    }
    const size_t pn_bytes = (size_t)P.kact * 4 * 8;
    rc = S.stage.ensure(P.o_pn + pn_bytes);
    if (rc) return rc;
    char *h = static_cast<char *>(S.stage.p);
    pack_values(lik, P, h);
    char *d = static_cast<char *>(P.prog.p);
    CXG_CUDA(cudaMemcpyAsync(d + P.o_elen, h + P.o_elen, P.o_dst - P.o_elen,
                             cudaMemcpyHostToDevice, S.stream));
    CXG_CUDA(cudaMemcpyAsync(d + P.o_pn, h + P.o_pn, pn_bytes, cudaMemcpyHostToDevice,
                             S.stream));
    CXG_CUDA(cudaEventRecord(S.stage_ev, S.stream));
    S.stage_pending = true;
    S.last_h2d = (P.o_dst - P.o_elen) + pn_bytes;
    P.pa.wnorm = lik->wNorm;
    P.a.freqs = static_cast<const uint32_t *>(dfreqs);
    return 0;
}

// Translate and run lik's plan.  `site` (host, mschars doubles) optional.
// A call whose plan has the key of the previous call's (the same steps on
// the same buffers, as a full re-plan of an unchanged tree gives) reuses
// that translation and uploads only the new values.
static int execute(CxtLik *lik, int prec, double *lnL, double *site) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    int rc = ensure_ready(S);
    if (rc) return rc;
    if (lik == nullptr) return fail(CXG_EINVAL, "lik is NULL");
    Plan &P = scratch_plan();
    static std::vector<uint64_t> key;
    plan_key(S, lik, prec, key);
    if (S.last_valid && key == S.last_key) {
        rc = refresh_values(S, lik, P);
    } else {
        S.last_valid = false;
        rc = translate(S, lik, prec, P, true, true);
        if (rc == 0) {
            plan_key(S, lik, prec, S.last_key);  // translating may allocate
            S.last_valid = true;
        }
    }
    if (rc) {
        S.last_valid = false;
        return rc;
    }
    rc = enqueue(S, P, site != nullptr, nullptr, nullptr, true);
    if (rc) {
        S.last_valid = false;
        return rc;
    }
    S.last_d2h = 32 + (site ? (size_t)P.npat * 8 : 0);
    rc = finish(S, P, lnL, site);
    if (rc) S.last_valid = false;
    return rc;
}

}  // namespace cxg

using namespace cxg;

extern "C" {

const char *cxgLastError(void) { return g_err.c_str(); }

int cxgInfo(char *buf, size_t len) {
    int dev = -1, rt = 0;
    cudaRuntimeGetVersion(&rt);
    cudaError_t e = cudaGetDevice(&dev);
    snprintf(buf, len, "cxlik_gpu 1 sm_103a cudart %d device %d%s", rt, dev,
             e == cudaSuccess ? "" : " (no device)");
    return 0;
}

int cxgLikClSetLeafMasks(const CxtLikCL *cl, const uint8_t *masks,
                         unsigned n) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    int rc = ensure_ready(S);
    if (rc) return rc;
    if (cl == nullptr || cl->cLMat == nullptr || masks == nullptr || n == 0)
        return fail(CXG_EINVAL, "cxgLikClSetLeafMasks: bad argument");
    return upload_leaf(S, cl->cLMat, masks, n, true);
}

int cxgLikClForget(const double *cLMat) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    auto it = S.cls.find((uintptr_t)cLMat);
    if (it != S.cls.end()) {
        free_cl(S, it->second);
        S.cls.erase(it);
        ++S.epoch;
    }
    return 0;
}

int cxgLikSetPatternWeights(const unsigned *freqs, unsigned n) {
    if (freqs == nullptr || n == 0)
        return fail(CXG_EINVAL, "cxgLikSetPatternWeights: NULL or empty weights");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    int rc = ensure_ready(S);
    if (rc) return rc;
    char key[64];
    snprintf(key, sizeof(key), "%p:%u", (const void *)freqs, n);
    FreqEntry &fe = S.freqs[key];
    rc = fe.dev.ensure((size_t)n * 4);
    if (rc) return rc;
    CXG_CUDA(cudaMemcpy(fe.dev.p, freqs, (size_t)n * 4, cudaMemcpyHostToDevice));
    fe.host.assign(freqs, freqs + n);
    fe.registered = true;
    return 0;
}

int cxgLikForgetPatternWeights(const unsigned *freqs, unsigned n) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    char key[64];
    snprintf(key, sizeof(key), "%p:%u", (const void *)freqs, n);
    auto it = S.freqs.find(key);
    if (it != S.freqs.end()) {
        if (it->second.dev.p) dev_free(it->second.dev.p);
        S.freqs.erase(it);
    }
    return 0;
}

int cxgLikReset(void) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    for (auto &kv : S.cls) free_cl(S, kv.second);
    S.cls.clear();
    ++S.epoch;
    S.last_valid = false;
    for (auto &kv : S.freqs)
        if (kv.second.dev.p) dev_free(kv.second.dev.p);
    S.freqs.clear();
    return 0;
}

int cxgTune(unsigned tile, unsigned tpp, unsigned ppt, size_t smem_budget) {
    if (tile != 32 && tile != 64 && tile != 128)
        return fail(CXG_EINVAL, "cxgTune: tile must be 32, 64 or 128");
    if (tpp != 1 && tpp != 2 && tpp != 4)
        return fail(CXG_EINVAL, "cxgTune: threads per pattern must be 1, 2 or 4");
    if (tile * tpp > kMaxThreads)
        return fail(CXG_EINVAL, "cxgTune: tile x threads per pattern above 256");
    if (ppt != 1 && ppt != 2)
        return fail(CXG_EINVAL, "cxgTune: patterns per thread must be 1 or 2");
    if (ppt == 2 && (tpp != 1 || tile < 64))
        return fail(CXG_EINVAL,
                    "cxgTune: two patterns per thread need one thread per pattern, tile >= 64");
    if (smem_budget > 200 * 1024)
        return fail(CXG_EINVAL, "cxgTune: shared-memory budget above 200 KiB");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    g_tile = tile;
    g_tpp = tpp;
    g_ppt = ppt;
    g_smem_budget = smem_budget;
    return 0;
}

int cxgTuneLanes(unsigned lanes) {
    if (lanes != 1 && lanes != 2)
        return fail(CXG_EINVAL, "cxgTuneLanes: op lanes must be 1 or 2");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    g_lanes = lanes;
    return 0;
}

int cxgTuneLanesGet(unsigned *lanes) {
    if (lanes) *lanes = g_lanes;
    return 0;
}

int cxgTuneGet(unsigned *tile, unsigned *tpp, unsigned *ppt, size_t *smem_budget) {
    if (tile) *tile = g_tile;
    if (tpp) *tpp = g_tpp;
    if (ppt) *ppt = g_ppt;
    if (smem_budget) *smem_budget = g_smem_budget;
    return 0;
}

int cxgDebugSetSpinLimit(unsigned limit, unsigned *previous) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    int rc = ensure_ready(S);
    if (rc) return rc;
    static unsigned current = kSpinLimit;
    // No walker of this library may be running while the bound changes.
    CXG_CUDA(device_sync());
    CXG_CUDA(set_spin_limit(limit));
    if (previous) *previous = current;
    current = limit;
    return 0;
}

int cxgDebugFailAllocs(long long after) {
    g_alloc_budget.store(after < 0 ? -1 : after);
    return 0;
}

int cxgDebugCanaries(int on) {
    g_canary_on.store(on ? 1 : 0);
    return 0;
}

int cxgDebugCanarySelfTest(int *detected) {
    if (detected == nullptr) return fail(CXG_EINVAL, "cxgDebugCanarySelfTest: NULL");
    if (!canary_on()) return fail(CXG_EINVAL, "cxgDebugCanarySelfTest: canaries are off");
    // A 1000-byte allocation whose canary a host-side memset then changes:
    // the byte written lies inside what cudaMalloc gave, past the 1000.
    void *p = nullptr;
    CXG_CUDA(dev_malloc(&p, 1000));
    CXG_CUDA(cudaMemset(static_cast<char *>(p) + 1000 + 17, 0, 1));
    CXG_CUDA(device_sync());
    size_t n = 0;
    {
        std::lock_guard<std::mutex> g(g_canary_mu);
        n = g_canary.count(p) ? g_canary[p] : 0;
    }
    *detected = (n == 1000 && !canary_intact(p, n)) ? 1 : 0;
    {
        std::lock_guard<std::mutex> g(g_canary_mu);
        g_canary.erase(p);
    }
    {
        std::lock_guard<std::mutex> gate(capture_gate());
        CXG_CUDA(cudaFree(p));
    }
    return 0;
}

int cxgDebugCheckCanaries(unsigned long long *checked, unsigned long long *bad) {
    CXG_CUDA(device_sync());
    std::vector<std::pair<void *, size_t>> live;
    {
        std::lock_guard<std::mutex> g(g_canary_mu);
        live.assign(g_canary.begin(), g_canary.end());
    }
    unsigned long long nbad = g_canary_bad.exchange(0);
    for (auto &kv : live)
        if (!canary_intact(kv.first, kv.second)) ++nbad;
    if (checked) *checked = live.size();
    if (bad) *bad = nbad;
    return 0;
}

int cxgLikLastIo(size_t *h2d, size_t *d2h) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    if (h2d) *h2d = S.last_h2d;
    if (d2h) *d2h = S.last_d2h;
    return 0;
}

int cxgLikDeviceBytes(size_t *bytes) {
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    if (bytes) *bytes = S.cl_bytes;
    return 0;
}

int cxgLikExecuteLnL(CxtLik *lik, int precision, double *lnL,
                     double *siteLnL) {
    NvtxRange r("cxgLikExecuteLnL");
    return execute(lik, precision, lnL, siteLnL);
}

struct cxgPlan {
    Plan p;
};

int cxgPlanCreate(CxtLik *lik, int precision, cxgPlan **out) {
    if (out == nullptr) return fail(CXG_EINVAL, "cxgPlanCreate: out is NULL");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    int rc = ensure_ready(S);
    if (rc) return rc;
    cxgPlan *h = new cxgPlan();
    rc = translate(S, lik, precision, h->p, true, true);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return 0;
}

int cxgPlanRun(cxgPlan *h, double *lnL, double *siteLnL) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgPlanRun: NULL plan");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    int rc = enqueue(S, h->p, siteLnL != nullptr);
    if (rc) return rc;
    return finish(S, h->p, lnL, siteLnL);
}

int cxgPlanTime(cxgPlan *h, int iters, double *ms_per_run,
                double *plan_kernel_ms, double *lnL) {
    if (h == nullptr || iters < 1) return fail(CXG_EINVAL, "cxgPlanTime: bad args");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    Plan &P = h->p;
    std::vector<cudaEvent_t> ev(2 * (size_t)iters + 2, nullptr);
    for (auto &e : ev) CXG_CUDA(cudaEventCreate(&e));
    int rc = 0;
    cudaError_t ce = cudaEventRecord(ev[0], S.stream);
    for (int i = 0; i < iters && rc == 0 && ce == cudaSuccess; ++i)
        rc = enqueue(S, P, false, ev[2 + 2 * i], ev[3 + 2 * i]);
    if (rc == 0 && ce == cudaSuccess) ce = cudaEventRecord(ev[1], S.stream);
    if (rc == 0 && ce == cudaSuccess) ce = cudaEventSynchronize(ev[1]);
    double kern = 0.0;
    float tot = 0.0f;
    if (rc == 0 && ce == cudaSuccess) {
        ce = cudaEventElapsedTime(&tot, ev[0], ev[1]);
        for (int i = 0; i < iters && ce == cudaSuccess; ++i) {
            float k = 0.0f;
            ce = cudaEventElapsedTime(&k, ev[2 + 2 * i], ev[3 + 2 * i]);
            kern += k;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "cxgPlanTime events");
    if (ms_per_run) *ms_per_run = tot / iters;
    if (plan_kernel_ms) *plan_kernel_ms = kern / iters;
    return finish(S, P, lnL, nullptr);
}

int cxgPlanShape(const cxgPlan *h, unsigned *tile, unsigned *tpp, unsigned *ppt,
                 unsigned *nslot, unsigned *nleaf) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgPlanShape: NULL plan");
    if (tile) *tile = h->p.tile;
    if (tpp) *tpp = h->p.tpp;
    if (ppt) *ppt = h->p.ppt;
    if (nslot) *nslot = h->p.nslot;
    if (nleaf) *nleaf = h->p.nleaf;
    return 0;
}

int cxgPlanLanes(const cxgPlan *h, unsigned *lanes) {
    if (h == nullptr || lanes == nullptr) return fail(CXG_EINVAL, "cxgPlanLanes: NULL argument");
    *lanes = h->p.lanes;
    return 0;
}

int cxgPlanInfo(const cxgPlan *h, double *updates, double *alg_bytes,
                unsigned *nops, unsigned *kernels_per_run) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgPlanInfo: NULL plan");
    if (updates) *updates = h->p.updates;
    if (alg_bytes) *alg_bytes = h->p.alg_bytes;
    if (nops) *nops = h->p.nops;
    if (kernels_per_run) *kernels_per_run = 2;
    return 0;
}

int cxgPlanDestroy(cxgPlan *h) {
    if (h == nullptr) return 0;
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    cudaStreamSynchronize(S.stream);
    free_plan(h->p);
    delete h;
    return 0;
}

// ---------------------------------------------------------------------------
// Batches: many translated plans run by one persistent launch.
// ---------------------------------------------------------------------------
struct cxgBatch {
    int prec = CXG_FP64;
    bool per_node = false;
    std::vector<Plan *> plans;
    DevBuf jobs, items, pmats, prefix, results;
    HostBuf out;
    // Jobs that stage their leaves and jobs that stream them run as two
    // persistent launches (each walker is built for one of the two).
    BatchArgs args[2];
    unsigned grid[2] = {0, 0}, nitems = 0;
    uint32_t pmat_total = 0;
    double updates = 0.0, alg_bytes = 0.0;
    unsigned long long launches = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

static void free_batch(cxgBatch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (Plan *p : b->plans) {
        free_plan(*p);
        delete p;
    }
    for (DevBuf *d : {&b->jobs, &b->items, &b->pmats, &b->prefix, &b->results})
        if (d->p) dev_free(d->p);
    if (b->out.p) host_free(b->out.p);
    delete b;
}

// Enqueue one run of the batch.  e0/e1 (optional) bracket the walker.
static int batch_enqueue(State &S, cxgBatch *b, cudaEvent_t e0 = nullptr,
                         cudaEvent_t e1 = nullptr) {
    const size_t n = b->plans.size();
    CXG_CUDA(cudaMemsetAsync(b->results.p, 0, n * 32 + 32, S.stream));
    CXG_CUDA(launch_pmat_batch(static_cast<const PmatArgs *>(b->pmats.p),
                               static_cast<const uint32_t *>(b->prefix.p),
                               (uint32_t)n, b->pmat_total, S.stream));
    if (e0) CXG_CUDA(cudaEventRecord(e0, S.stream));
    if (!b->per_node) {
        for (int gi = 0; gi < 2; ++gi)
            if (b->args[gi].nitems)
                CXG_CUDA(launch_batch(b->prec, b->args[gi], b->grid[gi], S.stream));
    } else {
        // The plain comparison: one launch per node update.
        for (Plan *P : b->plans) {
            for (unsigned o = 0; o < P->nops; ++o) {
                PlanArgs a = P->a;
                a.rec = P->a.rec + (size_t)o * P->a.rstride;
                a.lrows = P->a.lrows + (size_t)o * P->a.lmax;
                a.nops = 1;
                a.no_root = (o + 1 < P->nops) ? 1u : 0u;
                a.root_last = (o + 1 < P->nops) ? 0u : P->a.root_last;
                CXG_CUDA(launch_plan(b->prec, a, S.stream));
            }
        }
    }
    if (e1) CXG_CUDA(cudaEventRecord(e1, S.stream));
    CXG_CUDA(cudaMemcpyAsync(b->out.p, b->results.p, n * 32,
                             cudaMemcpyDeviceToHost, S.stream));
    return 0;
}

static int batch_finish(State &S, cxgBatch *b, double *lnLs) {
    CXG_CUDA(cudaStreamSynchronize(S.stream));
    const char *o = static_cast<const char *>(b->out.p);
    for (size_t j = 0; j < b->plans.size(); ++j) {
        uint32_t ninf, err;
        double tot[2];
        memcpy(&ninf, o + j * 32 + 4, 4);
        memcpy(&err, o + j * 32 + 8, 4);
        memcpy(tot, o + j * 32 + 16, 16);
        for (DevCL *p : b->plans[j]->parents) p->computed = (err == 0);
        if (err)
            return fail(CXG_ETIMEOUT,
                        "batched walker: an op-record copy did not complete");
        if (lnLs) lnLs[j] = ninf ? -INFINITY : tot[0] + tot[1];
    }
    return 0;
}

void CxLikExecute(CxtLik *lik) {
    // CxLik.c:914-968: nothing to do for an empty plan.
    if (lik == nullptr || lik->stepsLen == 0) return;
    NvtxRange r("CxLikExecute");
    double tot = 0.0;
    if (execute(lik, CXG_FP64, &tot, lik->siteLnL + lik->cbase) != 0) {
        // No error channel in the reference signature: poison the outputs
        // so a caller cannot mistake them for a likelihood.
        for (unsigned s = 0; s < lik->nstripes; ++s) lik->stripeLnL[s] = NAN;
        return;
    }
    // Per-stripe sums in pattern order, as each reference worker does.
    for (unsigned s = 0; s < lik->nstripes; ++s) {
        double acc = 0.0;
        const unsigned c0 = s * lik->stripeWidth;
        for (unsigned c = c0; c < c0 + lik->stripeWidth && c < lik->mschars; ++c)
            acc += lik->siteLnL[lik->cbase + c];
        lik->stripeLnL[s] = acc;
    }
}

int cxgBatchCreate(CxtLik *const *liks, unsigned n, int precision,
                   unsigned flags, cxgBatch **out) {
    if (out == nullptr || liks == nullptr || n == 0)
        return fail(CXG_EINVAL, "cxgBatchCreate: bad arguments");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    int rc = ensure_ready(S);
    if (rc) return rc;
    cxgBatch *b = new cxgBatch();
    b->prec = precision;
    b->per_node = (flags & CXG_BATCH_PER_NODE) != 0;
    unsigned kact = 0;
    for (unsigned j = 0; j < n; ++j) {
        Plan *P = new Plan();
        b->plans.push_back(P);
        rc = translate(S, liks[j], precision, *P, !b->per_node);
        if (rc) {
            free_batch(b);
            return rc;
        }
        if (j == 0) kact = P->kact;
        if (P->kact != kact) {
            free_batch(b);
            return fail(CXG_EINVAL,
                        "cxgBatchCreate: jobs must share the number of active "
                        "components (group them by K)");
        }
        b->updates += P->updates;
        b->alg_bytes += P->alg_bytes;
        b->launches += P->nops;
    }
    // Per-job results live side by side: [ticket ninf err pad total] x n,
    // then the work counters of the two launches (16 bytes apart).
    if ((rc = b->results.ensure((size_t)n * 32 + 32)) ||
        (rc = b->out.ensure((size_t)n * 32)) ||
        (rc = b->jobs.ensure((size_t)n * sizeof(PlanArgs))) ||
        (rc = b->pmats.ensure((size_t)n * sizeof(PmatArgs))) ||
        (rc = b->prefix.ensure((size_t)(n + 1) * 4))) {
        free_batch(b);
        return rc;
    }
    std::vector<PlanArgs> jobs(n);
    std::vector<PmatArgs> pm(n);
    std::vector<uint32_t> prefix(n + 1, 0);
    std::vector<WalkItem> items;
    char *res = static_cast<char *>(b->results.p);
    for (unsigned j = 0; j < n; ++j) {
        PlanArgs a = b->plans[j]->a;
        a.ticket = (unsigned *)(res + (size_t)j * 32);
        a.ninf = (uint32_t *)(res + (size_t)j * 32 + 4);
        a.err = (uint32_t *)(res + (size_t)j * 32 + 8);
        a.total = (double *)(res + (size_t)j * 32 + 16);
        a.site = nullptr;
        b->plans[j]->a = a;
        jobs[j] = a;
        pm[j] = b->plans[j]->pa;
        prefix[j + 1] = prefix[j] + pm[j].nchild * pm[j].kact;
        for (unsigned t = 0; t < a.ntiles; ++t) items.push_back(WalkItem{j, t});
    }
    // Staged-leaf jobs first, then streamed ones (the two launches); each
    // group longest jobs first, so its persistent grid ends together.
    std::stable_sort(items.begin(), items.end(),
                     [&](const WalkItem &x, const WalkItem &y) {
                         const bool sx = jobs[x.job].lmax != 0, sy = jobs[y.job].lmax != 0;
                         if (sx != sy) return sy;
                         return jobs[x.job].nops > jobs[y.job].nops;
                     });
    b->nitems = (unsigned)items.size();
    b->pmat_total = prefix[n];
    if ((rc = b->items.ensure(items.size() * sizeof(WalkItem)))) {
        free_batch(b);
        return rc;
    }
    cudaError_t e;
    if ((e = cudaMemcpy(b->jobs.p, jobs.data(), n * sizeof(PlanArgs),
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->pmats.p, pm.data(), n * sizeof(PmatArgs),
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->prefix.p, prefix.data(), (n + 1) * 4,
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->items.p, items.data(), items.size() * sizeof(WalkItem),
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
        free_batch(b);
        return cuda_fail(e, "cxgBatchCreate upload");
    }
    unsigned nstaged = 0;
    while (nstaged < items.size() && jobs[items[nstaged].job].lmax == 0) ++nstaged;
    for (int gi = 0; gi < 2; ++gi) {
        BatchArgs &ba = b->args[gi];
        memset(&ba, 0, sizeof(ba));
        const unsigned i0 = gi == 0 ? 0 : nstaged;
        const unsigned i1 = gi == 0 ? nstaged : (unsigned)items.size();
        ba.jobs = static_cast<const PlanArgs *>(b->jobs.p);
        ba.items = static_cast<const WalkItem *>(b->items.p) + i0;
        ba.nitems = i1 - i0;
        ba.counter = (unsigned *)(res + (size_t)n * 32 + 16 * gi);
        ba.tile = b->plans[0]->tile;
        ba.tpp = b->plans[0]->tpp;
        ba.ppt = b->plans[0]->ppt;
        ba.ring = kRing;
        ba.kact = kact;
        ba.max_rstride = 16;
        for (unsigned i = i0; i < i1; ++i) {
            const PlanArgs &a = jobs[items[i].job];
            ba.max_nslot = std::max(ba.max_nslot, a.nslot);
            ba.max_rstride = std::max(ba.max_rstride, a.rstride);
            ba.max_lmax = std::max(ba.max_lmax, a.lmax);
            ba.max_nleaf = std::max(ba.max_nleaf, a.nleaf);
        }
    }
    if (!b->per_node) {
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        b->launches = 0;
        for (int gi = 0; gi < 2; ++gi) {
            const BatchArgs &ba = b->args[gi];
            if (ba.nitems == 0) continue;
            const size_t smem =
                plan_smem_bytes(precision, kact, ba.tile, ba.max_nslot, kRing,
                                ba.max_rstride, ba.max_lmax, ba.max_nleaf);
            const int per =
                batch_ctas_per_sm(precision, kact, ba.tile, ba.tpp, ba.ppt, gi == 0, smem);
            if (per <= 0 || nsm <= 0) {
                free_batch(b);
                return fail(CXG_EINVAL, "cxgBatchCreate: walker does not fit an SM");
            }
            b->grid[gi] = (unsigned)(per * nsm);
            b->launches += 1;
        }
        // Capture one run as a CUDA graph.
        cudaGraph_t graph = nullptr;
        bool began = false;
        {
            std::lock_guard<std::mutex> gate(capture_gate());
            e = cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                began = true;
                rc = batch_enqueue(S, b);
                e = cudaStreamEndCapture(S.stream, &graph);
            }
        }
        if (!began) {
            free_batch(b);
            return cuda_fail(e, "cudaStreamBeginCapture");
        }
        if (rc || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            free_batch(b);
            return rc ? rc : cuda_fail(e, "cudaStreamEndCapture");
        }
        b->graph = graph;
        if ((e = cudaGraphInstantiate(&b->exec, graph, 0)) != cudaSuccess) {
            free_batch(b);
            return cuda_fail(e, "cudaGraphInstantiate");
        }
    } else {
        b->launches += 0;
    }
    *out = b;
    return 0;
}

int cxgBatchRun(cxgBatch *b, double *lnLs) {
    if (b == nullptr) return fail(CXG_EINVAL, "cxgBatchRun: NULL batch");
    NvtxRange r("cxgBatchRun");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    if (b->exec)
        CXG_CUDA(cudaGraphLaunch(b->exec, S.stream));
    else {
        int rc = batch_enqueue(S, b);
        if (rc) return rc;
    }
    return batch_finish(S, b, lnLs);
}

int cxgBatchTime(cxgBatch *b, int iters, double *ms_per_run,
                 double *walk_ms) {
    if (b == nullptr || iters < 1) return fail(CXG_EINVAL, "cxgBatchTime: bad args");
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    std::vector<cudaEvent_t> ev(2 * (size_t)iters + 2, nullptr);
    for (auto &x : ev) CXG_CUDA(cudaEventCreate(&x));
    int rc = 0;
    cudaError_t ce = cudaEventRecord(ev[0], S.stream);
    // Wall time per run through the graph (or the per-node launches).
    for (int i = 0; i < iters && rc == 0 && ce == cudaSuccess; ++i) {
        if (b->exec)
            ce = cudaGraphLaunch(b->exec, S.stream);
        else
            rc = batch_enqueue(S, b);
    }
    if (rc == 0 && ce == cudaSuccess) ce = cudaEventRecord(ev[1], S.stream);
    // Walker-only time, with events around the walker launch(es).
    for (int i = 0; i < iters && rc == 0 && ce == cudaSuccess; ++i)
        rc = batch_enqueue(S, b, ev[2 + 2 * i], ev[3 + 2 * i]);
    if (rc == 0 && ce == cudaSuccess) ce = cudaStreamSynchronize(S.stream);
    float tot = 0.0f;
    double walk = 0.0;
    if (rc == 0 && ce == cudaSuccess) {
        ce = cudaEventElapsedTime(&tot, ev[0], ev[1]);
        for (int i = 0; i < iters && ce == cudaSuccess; ++i) {
            float k = 0.0f;
            ce = cudaEventElapsedTime(&k, ev[2 + 2 * i], ev[3 + 2 * i]);
            walk += k;
        }
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "cxgBatchTime events");
    if (ms_per_run) *ms_per_run = tot / iters;
    if (walk_ms) *walk_ms = walk / iters;
    return batch_finish(S, b, nullptr);
}

int cxgBatchInfo(const cxgBatch *b, double *updates, double *alg_bytes,
                 unsigned *nitems, unsigned *grid,
                 unsigned long long *launches_per_run) {
    if (b == nullptr) return fail(CXG_EINVAL, "cxgBatchInfo: NULL batch");
    if (updates) *updates = b->updates;
    if (alg_bytes) *alg_bytes = b->alg_bytes;
    if (nitems) *nitems = b->nitems;
    if (grid) *grid = b->grid[0] + b->grid[1];
    if (launches_per_run) *launches_per_run = b->launches + 1;  // + P kernel
    return 0;
}

int cxgBatchDestroy(cxgBatch *b) {
    if (b == nullptr) return 0;
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    cudaStreamSynchronize(S.stream);
    free_batch(b);
    return 0;
}

bool CxLikQDecomp(int n, double *RTri, double *PiDiag, double *PiDiagNorm,
                  double *qNorm, double *qEigVecCube, double *qEigVals) {
    if (n != 4) {
        set_error("CxLikQDecomp: only 4-state models are decomposed on the GPU");
        return true;
    }
    State &S = state();
    std::lock_guard<std::mutex> g(S.mu);
    if (ensure_ready(S)) return true;
    if (S.out.ensure(74 * 8 + 10 * 8)) return true;
    if (S.misc.ensure(32 + 128 * 8 + 84 * 8)) return true;
    double *h = static_cast<double *>(S.out.p);
    for (int i = 0; i < 6; ++i) h[i] = RTri[i];
    for (int i = 0; i < 4; ++i) h[6 + i] = PiDiag[i];
    double *din = (double *)((char *)S.misc.p + 32);
    double *dout = din + 10;
    if (cudaMemcpyAsync(din, h, 10 * 8, cudaMemcpyHostToDevice, S.stream) !=
            cudaSuccess ||
        launch_qdecomp(din, din + 6, dout, S.stream) != cudaSuccess ||
        cudaMemcpyAsync(h, dout, 74 * 8, cudaMemcpyDeviceToHost, S.stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(S.stream) != cudaSuccess) {
        set_error("CxLikQDecomp: CUDA failure");
        return true;
    }
    if (h[73] != 0.0) {
        set_error("CxLikQDecomp: eigensystem failed");
        return true;
    }
    for (int i = 0; i < 4; ++i) PiDiagNorm[i] = h[i];
    *qNorm = h[4];
    for (int i = 0; i < 64; ++i) qEigVecCube[i] = h[5 + i];
    for (int i = 0; i < 4; ++i) qEigVals[i] = h[69 + i];
    return false;
}

void CxLikPt(int n, double *P, double *qEigVecCube, double *qEigVals,
             double v) {
    double ex[32];
    if (n < 1 || n > 32) return;
    for (int k = 0; k < n; ++k) ex[k] = exp(qEigVals[k] * v);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double p = 0.0;
            for (int k = 0; k < n; ++k) p += qEigVecCube[i * n * n + j * n + k] * ex[k];
            P[i * n + j] = p < 0.0 ? 0.0 : p;
        }
}

}  // extern "C"
