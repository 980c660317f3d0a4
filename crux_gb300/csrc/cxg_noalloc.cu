// cxgLikExecuteNoAlloc: the plan walker for callers that cannot allocate.
//
// Some callers own every byte of device memory themselves. A host
// application may reserve the GPU heap in its own pool or a framework's
// caching allocator. A latency-critical loop must not stall the device on
// cudaMalloc/cudaFree, which can synchronise. Such callers cannot let the
// library allocate device buffers on their behalf.
//
// This entry point evaluates one plan using only memory the caller passes
// (CL buffers, leaf masks, pattern weights, an optional site-lnL output)
// and a fixed scratch area: the file-scope array below.  It calls no
// cudaMalloc, cudaFree, cudaHostAlloc or stream/event creation, and no
// library routine that allocates.  The host side packs into a static host
// buffer.  The walker is the same as cxgLikExecuteLnL's, so results agree
// with that entry point to rounding.
//
// Limits (checked; larger inputs are rejected with CXG_EINVAL):
//   node updates (ops) <= 1024, children <= 2048, patterns <= 2^20,
//   active components <= 8, op records <= 1.5 MiB, FP64 leaf tables
//   <= 1.5 MiB.  The scratch array is 4 MiB, held by every GPU that loads
//   the library until the process exits.
//
// The scratch array is shared by every call: each call overwrites it,
// clears the counters that must start at zero, and reads its result back
// before returning.  Calls that overlap on the GPU, from several threads
// or on several streams, race on it; a mutex serialises calls from this
// process up to the point where the result has been read back.
#include <cuda_runtime.h>

#include <algorithm>
#include <math.h>
#include <string.h>

#include <mutex>

#include "cxg_internal.h"

namespace cxg {

constexpr size_t kNaScratchBytes = 4u << 20;
constexpr unsigned kNaMaxOps = 1024;
constexpr unsigned kNaMaxKids = 2048;
constexpr unsigned kNaMaxPatterns = 1u << 20;
constexpr size_t kNaRecBudget = 1536u << 10;
constexpr size_t kNaTabBudget = 1536u << 10;
constexpr unsigned kNaMaxDevices = 64;

// The device scratch.  Host code must not use &g_na_scratch as a device
// address: it names a host-side stand-in.  na_setup() asks the runtime for
// the device address once per device.
static __device__ __align__(256) unsigned char g_na_scratch[kNaScratchBytes];

static void *g_na_dev[kNaMaxDevices];
static unsigned char g_na_host[kNaScratchBytes];  // packing area (static)
static unsigned char g_na_result[32];
static std::mutex g_na_mu;

// Device address of the scratch array on the current device; the first call
// per device looks it up (do that first call before any stream capture).
// The address stays valid for the life of the device's primary context.
static int na_setup(unsigned char **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= (int)kNaMaxDevices)
        return fail(CXG_EINVAL, "device ordinal above 63");
    if (g_na_dev[dev] == nullptr) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
        g_na_dev[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_na_dev[dev]);
    return 0;
}

static size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

}  // namespace cxg

using namespace cxg;

extern "C" int cxgLikExecuteNoAlloc(const CxtLik *lik, int precision,
                                    const uint32_t *dFreqs, double *dSiteLnL,
                                    void *stream, double *lnL) {
    std::lock_guard<std::mutex> g(g_na_mu);
    if (lik == nullptr || dFreqs == nullptr || lnL == nullptr)
        return fail(CXG_EINVAL, "cxgLikExecuteNoAlloc: NULL argument");
    if (lik->dim != 4)
        return fail(CXG_EINVAL, "only 4-state (DNA) likelihoods run on the GPU");
    if (precision != CXG_FP64 && precision != CXG_FP32)
        return fail(CXG_EINVAL, "unknown precision");
    const unsigned npat = lik->mschars;
    if (npat == 0 || npat > kNaMaxPatterns)
        return fail(CXG_EINVAL, "cxgLikExecuteNoAlloc: patterns must be 1..2^20");
    const unsigned ppad = pad_patterns(npat);
    const int prec = precision;
    unsigned char *dev = nullptr;
    int rc = na_setup(&dev);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // Active components and their models (at most 8 of each).
    unsigned act[kMaxComps];
    unsigned kact = 0;
    for (unsigned mc = 0; mc < lik->compsLen; ++mc)
        if (lik->comps[mc].weightScaled != 0.0) {
            if (kact == kMaxComps)
                return fail(CXG_EINVAL, "more than 8 active mixture components");
            act[kact++] = mc;
        }
    if (kact == 0) return fail(CXG_EINVAL, "no component has non-zero weight");
    const CxtLikModel *models[kMaxComps];
    int32_t model_of[kMaxComps];
    unsigned nmod = 0;
    for (unsigned k = 0; k < kact; ++k) {
        const CxtLikModel *m = lik->comps[act[k]].model;
        int idx = -1;
        for (unsigned i = 0; i < nmod; ++i)
            if (models[i] == m) idx = (int)i;
        if (idx < 0) {
            idx = (int)nmod;
            models[nmod++] = m;
        }
        model_of[k] = idx;
    }

    // Pass 1: count ops and children, check the step grammar, and size the
    // records: each op's exact bytes (header, children, each child's area
    // by kind) and its number of leaf children, as the allocating path
    // sizes them.
    unsigned nops = 0, nkids = 0, maxdeg = 0, deg = 0;
    const CxtLikCL *cur = nullptr;
    unsigned expect = 0;
    size_t op_bytes = 0, max_bytes = 0;
    unsigned op_leaves = 0, lmax = 0;
    for (unsigned s = 0; s < lik->stepsLen; ++s) {
        const CxtLikStep &stp = lik->steps[s];
        if ((unsigned)stp.variant > 3) return fail(CXG_EINVAL, "bad step variant");
        const bool compute = stp.variant == CxeLikStepComputeL ||
                             stp.variant == CxeLikStepComputeI;
        const bool leaf = stp.variant == CxeLikStepComputeL ||
                          stp.variant == CxeLikStepMergeL;
        if (compute) {
            if (cur != nullptr)
                return fail(CXG_EINVAL, "Compute step before ntrail reached 0");
            cur = stp.parentCL;
            ++nops;
            deg = 0;
            op_bytes = sizeof(RecHead);
            op_leaves = 0;
        } else if (cur == nullptr || stp.parentCL != cur ||
                   stp.ntrail + 1 != expect) {
            return fail(CXG_EINVAL, "Merge step does not continue its node");
        }
        if (stp.parentCL == nullptr || stp.parentCL->cLMat == nullptr ||
            stp.parentCL->lnScale == nullptr || stp.childCL == nullptr ||
            stp.childCL->cLMat == nullptr)
            return fail(CXG_EINVAL, "step CL without device buffers");
        // CL rows move in 16-byte units.
        if (((uintptr_t)stp.parentCL->cLMat | (uintptr_t)stp.childCL->cLMat) % 16)
            return fail(CXG_EINVAL, "CL buffer not 16-byte aligned");
        ++nkids;
        if (++deg > maxdeg) maxdeg = deg;
        op_bytes += sizeof(RecChild) + child_area_bytes(prec, kact, leaf);
        if (leaf) ++op_leaves;
        expect = stp.ntrail;
        if (stp.ntrail == 0) {
            cur = nullptr;
            max_bytes = std::max(max_bytes, al16(op_bytes));
            lmax = std::max(lmax, op_leaves);
        }
    }
    if (cur != nullptr) return fail(CXG_EINVAL, "plan ends mid-node");
    if (nops > kNaMaxOps || nkids > kNaMaxKids)
        return fail(CXG_EINVAL, "cxgLikExecuteNoAlloc: more than 1024 node "
                                "updates or 2048 children");
    if (maxdeg > kMaxChildren) return fail(CXG_EINVAL, "node degree above 16");
    if (lik->rootCLC == nullptr || lik->rootCLC->cLMat == nullptr ||
        lik->rootCLC->lnScale == nullptr)
        return fail(CXG_EINVAL, "rootCLC without device buffers");
    if ((uintptr_t)lik->rootCLC->cLMat % 16)
        return fail(CXG_EINVAL, "CL buffer not 16-byte aligned");

    // Record stride: the largest op's own bytes.
    const size_t rstride = std::max<size_t>(16, max_bytes);
    if ((size_t)(nops ? nops : 1) * rstride > kNaRecBudget)
        return fail(CXG_EINVAL, "cxgLikExecuteNoAlloc: op records above 1.5 MiB");

    // Scratch layout (same offsets on host and device):
    //   misc 256 | records | elen | cmult | rmult | model | cube | eig | dst |
    //   tab | pn | leaf rows | ltab | partial
    const size_t o_misc = 0;
    const size_t o_rec = 256;
    const size_t o_elen = al16(o_rec + (size_t)(nops ? nops : 1) * rstride);
    const size_t o_cm = al16(o_elen + (size_t)nkids * 8);
    const size_t o_rm = al16(o_cm + kact * 8);
    const size_t o_mod = al16(o_rm + kact * 8);
    const size_t o_cube = al16(o_mod + kact * 4);
    const size_t o_eig = al16(o_cube + nmod * 64 * 8);
    const size_t o_dst = al16(o_eig + nmod * 4 * 8);
    const size_t o_tab = al16(o_dst + (size_t)nkids * 8);
    const size_t o_pn = al16(o_tab + (size_t)nkids * 4);
    // Leaf rows: up to lmax leaf children per op, null-terminated when
    // fewer.
    const size_t o_lrow = al16(o_pn + kact * 4 * 8);
    const size_t o_ltab =
        al16(o_lrow + (size_t)(nops ? nops : 1) * (lmax ? lmax : 1) * sizeof(void *));
    size_t ltab_bytes = 0;
    if (prec == CXG_FP64) {
        unsigned nleafkids = 0;
        for (unsigned s = 0; s < lik->stepsLen; ++s)
            if (lik->steps[s].variant == CxeLikStepComputeL ||
                lik->steps[s].variant == CxeLikStepMergeL)
                ++nleafkids;
        ltab_bytes = (size_t)nleafkids * 16 * kact * 4 * 8;
        if (ltab_bytes > kNaTabBudget)
            return fail(CXG_EINVAL, "cxgLikExecuteNoAlloc: leaf tables above 1.5 MiB");
    }
    const size_t o_part = al16(o_ltab + (ltab_bytes ? ltab_bytes : 16));
    unsigned tile = kTile;
    size_t budget = 0;
    {
        unsigned tpp_q = 1;
        unsigned ppt_q = 1;
        cxgTuneGet(&tile, &tpp_q, &ppt_q, &budget);
    }
    const unsigned tpp = tuned_tpp(prec, kact, tile);
    const unsigned nb = plan_blocks(ppad, tile);
    if (o_part + (size_t)nb * 16 > kNaScratchBytes)
        return fail(CXG_EINVAL, "cxgLikExecuteNoAlloc: scratch too small");
    const size_t upload = o_ltab;  // host-packed prefix (misc..root weights)

    unsigned char *h = g_na_host;
    memset(h, 0, upload);  // ticket, ninf, err and records start at zero

    // Pass 2: records and children.  Each op's parent is the CxtLikCL of
    // its Compute step; every pointer is the caller's device memory (a leaf
    // child's cLMat is its mask array, read directly by the walker).
    const CxtLikCL *op_parent[kNaMaxOps];
    int op_slot[kNaMaxOps];
    // Shared-memory stack slots (LIFO, oldest holder loses its slot), as in
    // the allocating path.
    // (Leaves always stream here: no leaf table in the fixed scratch.)
    const size_t base_b =
        plan_smem_bytes(prec, kact, tile, 0, kRing, (unsigned)rstride, lmax, 0);
    const size_t slot_b =
        plan_smem_bytes(prec, kact, tile, 1, kRing, (unsigned)rstride, lmax, 0) - base_b;
    const void **lrows = reinterpret_cast<const void **>(h + o_lrow);
    int owner[kMaxSlots];
    for (unsigned k = 0; k < kMaxSlots; ++k) owner[k] = -1;
    unsigned used = 0;
    unsigned o = 0, kid = 0, ntab = 0;
    unsigned cap = 0;
    if (budget > base_b) cap = (unsigned)((budget - base_b) / slot_b);
    if (cap > kMaxSlots) cap = kMaxSlots;
    uint64_t *dsts = reinterpret_cast<uint64_t *>(h + o_dst);
    int32_t *tabs = reinterpret_cast<int32_t *>(h + o_tab);
    double *elens = reinterpret_cast<double *>(h + o_elen);
    unsigned s = 0;
    while (s < lik->stepsLen) {
        // One op: steps s .. s+n-1.
        unsigned n = 1;
        while (lik->steps[s + n - 1].ntrail != 0) ++n;
        const CxtLikCL *par = lik->steps[s].parentCL;
        unsigned char *r = h + o_rec + (size_t)o * rstride;
        RecHead hd;
        memset(&hd, 0, sizeof(hd));
        hd.data = par->cLMat;
        hd.scaler = par->lnScale;
        hd.nchild = n;
        hd.slot = -1;
        size_t area = sizeof(RecHead) + n * sizeof(RecChild);
        for (unsigned ci = 0; ci < n; ++ci, ++kid) {
            const CxtLikStep &stp = lik->steps[s + ci];
            const bool leaf = stp.variant == CxeLikStepComputeL ||
                              stp.variant == CxeLikStepMergeL;
            RecChild ch;
            memset(&ch, 0, sizeof(ch));
            ch.data = stp.childCL->cLMat;
            ch.scaler = stp.childCL->lnScale;
            if (leaf) {
                // Mask rows are copied in tile-sized pieces: 16-byte aligned.
                if ((uintptr_t)stp.childCL->cLMat % 16)
                    return fail(CXG_EINVAL, "leaf mask array not 16-byte aligned");
                const void **lr = lrows + (size_t)o * lmax;
                unsigned j = 0;
                while (lr[j] != nullptr) ++j;
                lr[j] = stp.childCL->cLMat;
                ch.src = SRC_LEAF;
                ch.tab = prec == CXG_FP64 ? ntab : 0;
                tabs[kid] = prec == CXG_FP64 ? (int32_t)ntab++ : 0;
            } else {
                if (stp.childCL->lnScale == nullptr)
                    return fail(CXG_EINVAL, "internal child without scaler buffer");
                ch.src = SRC_GLOBAL;
                tabs[kid] = -1;
                // Produced earlier in this plan and still in its slot?
                for (int j = (int)o - 1; j >= 0; --j) {
                    if (op_parent[j] != stp.childCL) continue;
                    const int sl = op_slot[j];
                    if (sl >= 0 && owner[sl] == j) {
                        ch.src = SRC_SLOT;
                        ch.idx = (uint32_t)sl;
                        owner[sl] = -1;
                    }
                    break;
                }
            }
            const size_t ab = child_area_bytes(prec, kact, leaf);
            if (area + ab > rstride)
                return fail(CXG_EINVAL, "internal: child area outside its record");
            ch.off = (uint32_t)area;
            memcpy(r + sizeof(RecHead) + ci * sizeof(RecChild), &ch, sizeof(ch));
            // Byte offset from the start of the records (pa.rec).
            dsts[kid] = (size_t)o * rstride + area;
            area += ab;
            elens[kid] = stp.edgeLen;
        }
        op_parent[o] = par;
        op_slot[o] = -1;
        if (o + 1 < nops && cap > 0) {
            int sl = -1;
            for (unsigned k = 0; k < cap && sl < 0; ++k)
                if (owner[k] < 0) sl = (int)k;
            if (sl < 0) {
                int oldest = 0;
                for (unsigned k = 1; k < cap; ++k)
                    if (owner[k] < owner[oldest]) oldest = (int)k;
                sl = oldest;
            }
            owner[sl] = (int)o;
            op_slot[o] = sl;
            hd.slot = sl;
            if ((unsigned)sl + 1 > used) used = (unsigned)sl + 1;
        }
        if (prec == CXG_FP32 && n == 2) {
            RecChild k0, k1;
            memcpy(&k0, r + sizeof(RecHead), sizeof(k0));
            memcpy(&k1, r + sizeof(RecHead) + sizeof(RecChild), sizeof(k1));
            hd.flags |= op_kind_flags(k0.src, k0.data, k1.src, k1.data,
                                      o > 0 ? op_parent[o - 1]->cLMat : nullptr);
        }
        memcpy(r, &hd, sizeof(hd));
        ++o;
        s += n;
    }
    for (unsigned k = 0; k < kact; ++k) {
        const CxtLikComp &cp = lik->comps[act[k]];
        reinterpret_cast<double *>(h + o_cm)[k] = cp.cmult;
        reinterpret_cast<double *>(h + o_rm)[k] = cp.model->rmult;
        reinterpret_cast<int32_t *>(h + o_mod)[k] = model_of[k];
        for (unsigned i = 0; i < 4; ++i)
            reinterpret_cast<double *>(h + o_pn)[k * 4 + i] =
                cp.model->piDiagNorm[i] * cp.weightScaled;
    }
    for (unsigned m = 0; m < nmod; ++m) {
        memcpy(h + o_cube + m * 64 * 8, models[m]->qEigVecCube, 64 * 8);
        memcpy(h + o_eig + m * 4 * 8, models[m]->qEigVals, 4 * 8);
    }
    const bool root_last =
        nops > 0 && op_parent[nops - 1] == lik->rootCLC;

    cudaError_t e = cudaMemcpyAsync(dev, h, upload, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(scratch)");

    PmatArgs pa;
    pa.nchild = nkids;
    pa.kact = kact;
    pa.precision = prec;
    pa.edge_len = reinterpret_cast<const double *>(dev + o_elen);
    pa.cmult = reinterpret_cast<const double *>(dev + o_cm);
    pa.rmult = reinterpret_cast<const double *>(dev + o_rm);
    pa.model = reinterpret_cast<const int32_t *>(dev + o_mod);
    pa.cube = reinterpret_cast<const double *>(dev + o_cube);
    pa.eig = reinterpret_cast<const double *>(dev + o_eig);
    pa.dst = reinterpret_cast<const uint64_t *>(dev + o_dst);
    pa.tab = reinterpret_cast<const int32_t *>(dev + o_tab);
    pa.wnorm = lik->wNorm;
    pa.wnorm_dev = nullptr;
    pa.rec = dev + o_rec;
    pa.ltab = reinterpret_cast<double *>(dev + o_ltab);
    e = launch_pmat(pa, st);
    if (e != cudaSuccess) return cuda_fail(e, "pmat_kernel");

    PlanArgs a;
    memset(&a, 0, sizeof(a));
    a.rec = dev + o_rec;
    a.lrows = reinterpret_cast<const uint8_t *const *>(dev + o_lrow);
    a.lmax = lmax;
    a.rstride = (uint32_t)rstride;
    a.ring = kRing;
    a.nops = nops;
    a.nslot = used;
    a.tile = tile;
    a.tpp = tpp;
    a.ppt = tuned_ppt(prec, kact, tile, tpp);
    a.kact = kact;
    a.npat = npat;
    a.ppad = ppad;
    a.root_last = root_last ? 1u : 0u;
    a.pn = reinterpret_cast<const double *>(dev + o_pn);
    a.root = lik->rootCLC->cLMat;
    a.rootsc = lik->rootCLC->lnScale;
    a.freqs = dFreqs;
    a.site = dSiteLnL;
    a.partial = reinterpret_cast<double *>(dev + o_part);
    a.ticket = reinterpret_cast<unsigned *>(dev + o_misc);
    a.ninf = reinterpret_cast<uint32_t *>(dev + o_misc + 4);
    a.err = reinterpret_cast<uint32_t *>(dev + o_misc + 8);
    a.total = reinterpret_cast<double *>(dev + o_misc + 16);
    a.ltab = reinterpret_cast<const double *>(dev + o_ltab);
    a.ntiles = nb;
    a.no_root = 0;
    e = launch_plan(prec, a, st);
    if (e != cudaSuccess) return cuda_fail(e, "walk_kernel");
    e = cudaMemcpyAsync(g_na_result, dev + o_misc, 32, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(result)");
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    uint32_t ninf, err;
    double tot[2];
    memcpy(&ninf, g_na_result + 4, 4);
    memcpy(&err, g_na_result + 8, 4);
    memcpy(tot, g_na_result + 16, 16);
    if (err)
        return fail(CXG_ETIMEOUT,
                    "plan walker: an op-record copy did not complete in time");
    *lnL = ninf ? -INFINITY : tot[0] + tot[1];
    return 0;
}
