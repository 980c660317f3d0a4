// Device kernels of the pruning likelihood on sm_103a.
//
// Layout in HBM: a CL buffer of K active components over ppad patterns is
// [K][U][ppad] 16-byte units (FP32: U = 1, a float4 of the four states;
// FP64: U = 2, two double2), so that the threads of a warp, one pattern
// each, move 512 contiguous bytes per instruction.  Leaves are one uint8
// state mask per pattern.  Scalers are one FP64 log scale (plain form) or
// one int32 power-of-two exponent (FP32 form) per pattern.
//
// Kernels:
//   pmat_kernel     P(t) = V diag(exp(lambda r t)) V^-1 per (child edge,
//                   component), FP64, clipped at 0 (CxLik.c:258-292), plus
//                   the 16-entry message table of every leaf child.
//   walk_kernel<T>  one CTA per tile of patterns, one thread per pattern,
//                   walks the whole node-update list (patterns are
//                   independent through the entire post-order,
//                   CxLik.c:314-596, so no grid-wide sync is needed).  CLs
//                   produced and consumed within the walk stay in a
//                   shared-memory stack (slots assigned by the host), so HBM
//                   sees the write-through of every parent, the staged leaf
//                   masks and CLs cached by earlier runs.  Then it
//                   aggregates the root (CxLik.c:598-632) and reduces the
//                   weighted site lnLs with a compensated sum.
//   qdecomp_kernel  FP64 eigensystem of a reversible 4x4 Q by Jacobi
//                   rotations of the symmetrised matrix (CxLik.c:59-250).
#include <math.h>

#include <mutex>

#include "cxg_internal.h"
#include "cxg_device.cuh"

namespace cxg {

// ---------------------------------------------------------------------------
// P matrices, written into the op records.
// ---------------------------------------------------------------------------
// Four lanes per (child edge, component), see pmat_one.
// Programmatic dependent launch: a walker launched as a dependent of the
// P kernel may start (be scheduled, set up its shared memory and barriers)
// once every P block has started; it waits here, before it copies its
// first records, for the P kernel's matrices and their memory.  Without
// such a dependency both instructions do nothing.
__device__ __forceinline__ void pdl_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__global__ void pmat_kernel(PmatArgs a) {
    pdl_launch_dependents();
    // The walker's result words (ticket, counts, sum): it reads them only
    // after this grid has completed (stream order, or griddepcontrol.wait).
    if (a.zero != nullptr && blockIdx.x == 0 && threadIdx.x < 4) a.zero[threadIdx.x] = 0;
    const unsigned idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    if (idx >= a.nchild * a.kact) return;  // the same for all four lanes
    pmat_one(a, idx, threadIdx.x & 3u);
}

// P matrices of many jobs in one launch: (edge, component) t belongs to
// the job whose prefix range [prefix[j], prefix[j+1]) holds it.
__global__ void pmat_batch_kernel(const PmatArgs *jobs, const uint32_t *prefix,
                                  uint32_t njobs, uint32_t total) {
    const unsigned t = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    if (t >= total) return;
    unsigned lo = 0, hi = njobs;  // find j with prefix[j] <= t < prefix[j+1]
    while (hi - lo > 1) {
        const unsigned mid = (lo + hi) / 2;
        if (prefix[mid] <= t) lo = mid; else hi = mid;
    }
    pmat_one(jobs[lo], t - prefix[lo], threadIdx.x & 3u);
}

cudaError_t launch_pmat_batch(const PmatArgs *jobs, const uint32_t *prefix,
                              uint32_t njobs, uint32_t total, cudaStream_t s) {
    if (total == 0) return cudaSuccess;
    pmat_batch_kernel<<<(total + 31) / 32, 128, 0, s>>>(jobs, prefix, njobs, total);
    return cudaGetLastError();
}

cudaError_t launch_pmat(const PmatArgs &a, cudaStream_t s) {
    const unsigned n = a.nchild * a.kact;
    if (n == 0) return cudaSuccess;
    pmat_kernel<<<(n + 31) / 32, 128, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Compensated (Neumaier two-sum) reduction helpers.
// ---------------------------------------------------------------------------
struct Comp {
    double s, c;
};

__device__ __forceinline__ Comp comp_add(Comp a, Comp b) {
    const double s = a.s + b.s;
    const double bb = s - a.s;
    const double err = (a.s - (s - bb)) + (b.s - bb);
    return Comp{s, a.c + b.c + err};
}

__device__ __forceinline__ Comp warp_comp(Comp v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Comp o;
        o.s = __shfl_down_sync(0xffffffffu, v.s, off);
        o.c = __shfl_down_sync(0xffffffffu, v.c, off);
        v = comp_add(v, o);
    }
    return v;
}

// Tile sum of site values (finite values; -inf sites are counted
// separately) into a.partial[tile]; the last tile of the job to finish
// folds all of the job's partials into a.total.  Thread t holds the values
// of patterns t + h * blockDim (h < NV): every group of 32 consecutive
// patterns reduces by the same shuffle tree and the groups add in pattern
// order, and warp 0 alone folds the partials, so the sums do not depend
// on the launch shape.
template <int NV>
__device__ void reduce_sites_n(const PlanArgs &a, unsigned tile_idx, const double *v,
                               const bool *neg_inf) {
    __shared__ Comp warp_part[2 * kMaxThreads / 32];
    __shared__ unsigned ninf_block;
    __shared__ bool last;
    const unsigned nwarp = blockDim.x / 32;
    if (threadIdx.x == 0) ninf_block = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int h = 0; h < NV; ++h) {
        if (neg_inf[h]) atomicAdd(&ninf_block, 1u);
        const Comp c = warp_comp(Comp{v[h], 0.0});
        if (lane == 0) warp_part[h * nwarp + warp] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp b = warp_part[0];
        for (unsigned w = 1; w < NV * nwarp; ++w) b = comp_add(b, warp_part[w]);
        a.partial[2 * tile_idx] = b.s;
        a.partial[2 * tile_idx + 1] = b.c;
        if (ninf_block) atomicAdd(a.ninf, ninf_block);
        __threadfence();
        const unsigned t = atomicAdd(a.ticket, 1u);
        last = (t == a.ntiles - 1);
    }
    __syncthreads();
    if (last && warp == 0) {
        __threadfence();
        Comp acc{0.0, 0.0};
        for (unsigned b = lane; b < a.ntiles; b += 32) {
            const volatile double *pp = a.partial;
            acc = comp_add(acc, Comp{pp[2 * b], pp[2 * b + 1]});
        }
        acc = warp_comp(acc);
        if (lane == 0) {
            a.total[0] = acc.s;
            a.total[1] = acc.c;
            *a.ticket = 0;  // ready for the next launch
        }
    }
    __syncthreads();  // warp_part / last are reused by the next item
}

__device__ __forceinline__ void reduce_sites(const PlanArgs &a, unsigned tile_idx, double v,
                                             bool neg_inf) {
    reduce_sites_n<1>(a, tile_idx, &v, &neg_inf);
}

// ---------------------------------------------------------------------------
// Plan walker.  T = double: plain form, the reference's scaler (max over
// child messages, CxLik.c:390-403 and 577-588).  T = float: FP32 form, scale
// by the power of two that puts the largest parent entry in [0.5, 1); the
// exponent is an exact integer.
// ---------------------------------------------------------------------------
template <typename T>
struct Prec;

template <>
struct Prec<double> {
    typedef double S;   // scaler type
    typedef double2 V;  // 16-byte unit
    static constexpr int U = 2;
};

template <>
struct Prec<float> {
    typedef int S;
    typedef float4 V;
    static constexpr int U = 1;
};

__device__ __forceinline__ void unpack(const float4 v, float *x) {
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ float4 pack4(const float *x) {
    return make_float4(x[0], x[1], x[2], x[3]);
}
__device__ __forceinline__ void unpack(const double2 v, double *x) {
    x[0] = v.x; x[1] = v.y;
}
__device__ __forceinline__ double2 pack2(const double *x) {
    return make_double2(x[0], x[1]);
}

// Four states of component k of a CL held as U units at `base` with unit
// stride `stride` (HBM: ppad; shared memory: tile).
template <typename T>
__device__ __forceinline__ void load4(const typename Prec<T>::V *base,
                                      size_t stride, T *x);
template <>
__device__ __forceinline__ void load4<float>(const float4 *base, size_t,
                                             float *x) {
    unpack(*base, x);
}
template <>
__device__ __forceinline__ void load4<double>(const double2 *base,
                                              size_t stride, double *x) {
    unpack(base[0], x);
    unpack(base[stride], x + 2);
}
template <typename T>
__device__ __forceinline__ void store4(typename Prec<T>::V *base,
                                       size_t stride, const T *x);
template <>
__device__ __forceinline__ void store4<float>(float4 *base, size_t,
                                              const float *x) {
    *base = pack4(x);
}
template <>
__device__ __forceinline__ void store4<double>(double2 *base, size_t stride,
                                               const double *x) {
    base[0] = pack2(x);
    base[stride] = pack2(x + 2);
}
// Read-only 16-byte load through the non-coherent path.
__device__ __forceinline__ float4 ldro(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ double2 ldro(const double2 *p) { return __ldg(p); }

__device__ __forceinline__ float pow2f(int n) {  // n in [-126, 127]
    return __int_as_float((n + 127) << 23);
}

// Shared memory of one CTA: mbarriers [ring]; the stage ring [ring] of
// `stage` bytes, each an op record (rstride) followed, for a job that
// streams its leaves, by this tile's mask rows of the op's leaf children
// (lmax rows of tile bytes); stack slots [nslot][K][U][tile] units; slot
// scalers [nslot][tile]; and, for a job that stages its leaves, every
// leaf's mask row [nleaf][tile], loaded once per tile.  A batched launch
// lays it out for its largest job; every job uses a prefix of each region.
struct SmemLayout {
    size_t bars, ring, stage, slots, slot_sc, masks, total;
};

static __host__ __device__ SmemLayout smem_layout(int precision, unsigned kact,
                                                  unsigned tile, unsigned nslot,
                                                  unsigned ring, unsigned rstride,
                                                  unsigned lmax, unsigned nleaf) {
    const size_t U = precision == CXG_FP32 ? 1 : 2;
    const size_t sc = precision == CXG_FP32 ? 4 : 8;
    SmemLayout L;
    L.bars = 0;
    L.ring = ((size_t)ring * 8 + 127) & ~(size_t)127;
    L.stage = ((size_t)rstride + (size_t)lmax * tile + 15) & ~(size_t)15;
    L.slots = L.ring + (size_t)ring * L.stage;
    L.slot_sc = L.slots + (size_t)nslot * kact * U * tile * 16;
    L.masks = L.slot_sc + (((size_t)nslot * tile * sc + 15) & ~(size_t)15);
    L.total = L.masks + (size_t)nleaf * tile;
    return L;
}

size_t plan_smem_bytes(int precision, unsigned kact, unsigned tile, unsigned nslot,
                       unsigned ring, unsigned rstride, unsigned lmax, unsigned nleaf) {
    return smem_layout(precision, kact, tile, nslot, ring, rstride, lmax, nleaf).total;
}

// --- mbarrier and bulk-copy primitives (PTX) --------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(count)
                 : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Leaf-row pointers of op q that thread 0 reads ahead (the first
// kLeafPre; rows past them are read when the stage is issued).  Indexed
// with constants only, so they stay in registers.
constexpr int kLeafPre = 4;
__device__ __forceinline__ void read_rows(const PlanArgs &a, unsigned q,
                                          const uint8_t *(&pre)[kLeafPre]) {
    const uint8_t *const *rows = a.lrows + (size_t)q * a.lmax;
#pragma unroll
    for (int j = 0; j < kLeafPre; ++j) pre[j] = (unsigned)j < a.lmax ? rows[j] : nullptr;
}

// Start op q's stage: its record and this tile's mask rows of its leaf
// children (a.lrows[q][0..lmax), null-terminated, in the record's child
// order), all completing on the stage's mbarrier.
__device__ __forceinline__ void issue_stage(const PlanArgs &a, unsigned q,
                                            unsigned char *st, uint64_t *bar,
                                            unsigned tile_idx, unsigned tile,
                                            const uint8_t *const (&pre)[kLeafPre]) {
    const uint8_t *const *rows = a.lrows + (size_t)q * a.lmax;
    unsigned n = 0;
#pragma unroll
    for (int j = 0; j < kLeafPre; ++j)
        if (n == (unsigned)j && pre[j] != nullptr) n = j + 1;
    if (n == kLeafPre)
        while (n < a.lmax && rows[n] != nullptr) ++n;
    fence_proxy_async();
    mbar_expect_tx(bar, a.rstride + n * tile);
    bulk_g2s(st, a.rec + (size_t)q * a.rstride, a.rstride, bar);
    const size_t off = (size_t)tile_idx * tile;
#pragma unroll
    for (int j = 0; j < kLeafPre; ++j)
        if ((unsigned)j < n) bulk_g2s(st + a.rstride + (size_t)j * tile, pre[j] + off, tile, bar);
    for (unsigned j = kLeafPre; j < n; ++j)
        bulk_g2s(st + a.rstride + (size_t)j * tile, rows[j] + off, tile, bar);
}

// Attempts of mbarrier.try_wait per record wait (set_spin_limit; the
// default is kSpinLimit, 0 gives up without waiting).  Read once per tile
// by the thread that waits.
__device__ uint32_t g_spin_limit = kSpinLimit;

cudaError_t set_spin_limit(uint32_t limit) {
    return cudaMemcpyToSymbol(g_spin_limit, &limit, sizeof(limit));
}

// Spin on a phase with an iteration bound; false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint32_t limit = kSpinLimit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// After a wait gave up at op (or step) o of n: wait, with the default
// bound, for the copies still in flight into the ring -- the stages of
// ops o .. o + R - 1 -- so that none lands after the CTA has left.
// `phase` is the parity state before op o's stage was flipped.
__device__ __noinline__ void drain_ring(uint64_t *bars, uint32_t phase, unsigned o,
                                        unsigned n, unsigned R) {
    for (unsigned q = o; q < n && q < o + R; ++q) {
        const unsigned st = q % R;
        mbar_wait_bounded(&bars[st], (phase >> st) & 1u);
    }
}

// The per-op hand-off barrier of the walkers: true when every thread's
// record wait succeeded.  `ok` is uniform within each warp.
__device__ __forceinline__ bool cta_hand_off(bool ok, unsigned nthr) {
    if (nthr == 32) {
        __syncwarp();
        return ok;
    }
    return __syncthreads_and(ok) != 0;
}

// Max of n values as a balanced tree (the same value as a left-to-right
// chain: fmax is exact and ignores NaN operands either way), so the
// dependent chain is log2(n) long instead of n.
template <int N, typename X>
__device__ __forceinline__ X tree_max(const X *v) {
    if constexpr (N == 1) {
        return v[0];
    } else {
        constexpr int H = N / 2;
        return fmax(tree_max<H>(v), tree_max<N - H>(v + H));
    }
}

// Max over the G consecutive lanes that share a pattern.
template <int G, typename X>
__device__ __forceinline__ X group_max(X x) {
#pragma unroll
    for (int o = 1; o < G; o <<= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

// The plain form's scaler: the max over child messages of doubles that are
// >= 0 (P entries are clamped at 0, CL rows are their products), taken on
// the bit patterns with integer compares, which order non-negative doubles
// as their values.  The value is fmax's, and the FP64 pipe, which bounds
// the plain form, does no max work.  (A NaN entry would win here where
// fmax skips it; a pattern with a NaN entry ends with a NaN site lnL
// either way, since the entry is in the parent's rows.)
__device__ __forceinline__ double max_nonneg(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x > y ? x : y);
}
template <int N>
__device__ __forceinline__ double tree_max_nonneg(const double *v) {
    if constexpr (N == 1) {
        return v[0];
    } else {
        constexpr int H = N / 2;
        return max_nonneg(tree_max_nonneg<H>(v), tree_max_nonneg<N - H>(v + H));
    }
}
template <int G>
__device__ __forceinline__ double group_max_nonneg(double x) {
#pragma unroll
    for (int o = 1; o < G; o <<= 1) x = max_nonneg(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

// --- FP32 two-child ops by kind (one thread per pattern) --------------------
// Row r of a P matrix against the four states x of one component, in the
// order of the general path (a product, then three fused adds).
__device__ __forceinline__ float pdot(const float4 r, const float *x) {
    float v = r.x * x[0];
    v = fmaf(r.y, x[1], v);
    v = fmaf(r.z, x[2], v);
    v = fmaf(r.w, x[3], v);
    return v;
}

// An internal child's rows and exponent: from its stack slot, or from HBM
// through L2 (the rows were written by this same thread earlier in the
// walk, or by an earlier launch).
template <int KT>
__device__ __forceinline__ int load_internal(const RecChild &c, const float4 *slots,
                                             const int *slot_sc, unsigned tile,
                                             unsigned pl, unsigned p, size_t ppad,
                                             float *x) {
    if (c.src == SRC_SLOT) {
        const float4 *s = slots + (size_t)c.idx * KT * tile + pl;
#pragma unroll
        for (int k = 0; k < KT; ++k) unpack(s[(size_t)k * tile], x + 4 * k);
        return slot_sc[(size_t)c.idx * tile + pl];
    }
    const float4 *g = static_cast<const float4 *>(c.data) + p;
#pragma unroll
    for (int k = 0; k < KT; ++k) unpack(__ldcg(g + (size_t)k * ppad), x + 4 * k);
    return __ldcg(static_cast<const int *>(c.scaler) + p);
}

// One two-child op of kind `kind` (OPK_*) for the NP patterns pl[h] (in
// the tile) / p[h] (in the CL buffers) a thread owns: acc[h] becomes the
// product of the two children's messages and lns[h] the sum of their
// exponents.  acc holds the previous op's result on entry (child A of the
// F kinds), with its exponents in lns.  `ia` is child A's record index; a
// streamed leaf's row is its rank among the op's leaf children.  Each P
// row is read from shared memory once for all NP patterns.
template <int KT, bool STAGED, int NP>
__device__ __forceinline__ void op2_kind(uint32_t kind, const unsigned char *rec,
                                         const RecChild *kids, unsigned ia,
                                         float (&acc)[NP][KT * 4], int (&lns)[NP],
                                         const uint8_t *masks, const uint8_t *lrow,
                                         const float4 *slots, const int *slot_sc,
                                         unsigned tile, const unsigned (&pl)[NP],
                                         const unsigned (&p)[NP], size_t ppad) {
    const RecChild &cA = kids[ia];
    const RecChild &cB = kids[ia ^ 1u];
    const float4 *PA = reinterpret_cast<const float4 *>(rec + cA.off);
    const float4 *PB = reinterpret_cast<const float4 *>(rec + cB.off);
    auto mask = [&](const RecChild &c, unsigned rank, unsigned q) -> unsigned {
        return STAGED ? masks[(size_t)c.idx * tile + q] : lrow[(size_t)rank * tile + q];
    };
    // y = a * b, one component (states 0..3) at a time.
    auto mul4 = [](float *y, const float *a, const float4 b) {
        y[0] = a[0] * b.x;
        y[1] = a[1] * b.y;
        y[2] = a[2] * b.z;
        y[3] = a[3] * b.w;
    };
    switch (kind) {
    case OPK_LL: {
        unsigned mA[NP], mB[NP];
#pragma unroll
        for (int h = 0; h < NP; ++h) {
            mA[h] = mask(cA, ia, pl[h]);
            mB[h] = mask(cB, ia ^ 1u, pl[h]);
        }
#pragma unroll
        for (int k = 0; k < KT; ++k)
#pragma unroll
            for (int h = 0; h < NP; ++h) {
                const float4 a = PA[k * 16 + mA[h]];
                const float ax[4] = {a.x, a.y, a.z, a.w};
                mul4(acc[h] + 4 * k, ax, PB[k * 16 + mB[h]]);
            }
#pragma unroll
        for (int h = 0; h < NP; ++h) lns[h] = 0;
        return;
    }
    case OPK_FL:
    case OPK_IL: {
        // A's rows: the previous result (FL) or loaded (IL); B a leaf.
        float xA[NP][KT * 4];
        int lA[NP];
#pragma unroll
        for (int h = 0; h < NP; ++h) {
            if (kind == OPK_IL) {
                lA[h] = load_internal<KT>(cA, slots, slot_sc, tile, pl[h], p[h], ppad, xA[h]);
            } else {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) xA[h][q] = acc[h][q];
                lA[h] = lns[h];
            }
        }
        unsigned mB[NP];
#pragma unroll
        for (int h = 0; h < NP; ++h) mB[h] = mask(cB, 0, pl[h]);
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            float m[NP][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float4 r = PA[k * 4 + i];
#pragma unroll
                for (int h = 0; h < NP; ++h) m[h][i] = pdot(r, xA[h] + 4 * k);
            }
#pragma unroll
            for (int h = 0; h < NP; ++h) mul4(acc[h] + 4 * k, m[h], PB[k * 16 + mB[h]]);
        }
#pragma unroll
        for (int h = 0; h < NP; ++h) lns[h] = lA[h];
        return;
    }
    case OPK_FI: {
        float xB[NP][KT * 4];
        int lB[NP];
#pragma unroll
        for (int h = 0; h < NP; ++h)
            lB[h] = load_internal<KT>(cB, slots, slot_sc, tile, pl[h], p[h], ppad, xB[h]);
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            float m[NP][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float4 r = PA[k * 4 + i];
#pragma unroll
                for (int h = 0; h < NP; ++h) m[h][i] = pdot(r, acc[h] + 4 * k);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float4 r = PB[k * 4 + i];
#pragma unroll
                for (int h = 0; h < NP; ++h) acc[h][4 * k + i] = m[h][i] * pdot(r, xB[h] + 4 * k);
            }
        }
#pragma unroll
        for (int h = 0; h < NP; ++h) lns[h] = lns[h] + lB[h];
        return;
    }
    default: {  // OPK_II
        float xA[NP][KT * 4], xB[NP][KT * 4];
        int lA[NP], lB[NP];
#pragma unroll
        for (int h = 0; h < NP; ++h) {
            lA[h] = load_internal<KT>(cA, slots, slot_sc, tile, pl[h], p[h], ppad, xA[h]);
            lB[h] = load_internal<KT>(cB, slots, slot_sc, tile, pl[h], p[h], ppad, xB[h]);
        }
#pragma unroll
        for (int k = 0; k < KT; ++k)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float4 ra = PA[k * 4 + i], rb = PB[k * 4 + i];
#pragma unroll
                for (int h = 0; h < NP; ++h)
                    acc[h][4 * k + i] = pdot(ra, xA[h] + 4 * k) * pdot(rb, xB[h] + 4 * k);
            }
#pragma unroll
        for (int h = 0; h < NP; ++h) lns[h] = lA[h] + lB[h];
        return;
    }
    }
}

// Walk every op of job `a` for tile `tile_idx`, aggregate the root and
// reduce.  G consecutive threads share a pattern, each holding KT of its
// KT*G components; with G = 1 one thread owns a pattern.  Every G gives the
// same bits: scalers are maxima over the group, and the root sum and the
// tile reduction run in the G = 1 order.  `phase` (thread 0 only) holds,
// per ring stage, the parity of the next completion to wait for; it
// persists across the items a CTA processes.  Returns false if a bounded
// wait gave up.
//
// L > 1 (op lanes; FP32, G = 1, staged leaves): the CTA is L groups of
// `tile` threads over the same patterns.  The host schedules the plan in
// steps of L mutually independent ops (a record with no children fills an
// empty lane) and a ring stage holds one step's L records; lane l runs the
// step's l-th op.  A result one lane writes is read by another only in a
// later step, after the block barriers between steps.  The root is the
// last step's lane-0 op, so lane 0 aggregates it and the other lanes add
// exact zeros to the tile sum: the bits are those of L = 1.
template <typename T, int KT, int G, bool STAGED, int L = 1>
__device__ bool walk_tile(const PlanArgs &a, unsigned tile_idx,
                          const SmemLayout &Lay, unsigned ring_depth,
                          uint32_t &phase) {
    static_assert(L == 1 || (STAGED && G == 1 && sizeof(T) == 4),
                  "op lanes: FP32, one thread per pattern, staged leaves");
    typedef typename Prec<T>::S S;
    typedef typename Prec<T>::V V;
    constexpr int U = Prec<T>::U;
    constexpr int KA = KT * G;  // active components of the job
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned nthr = blockDim.x;
    const unsigned tile = nthr / (G * L);
    const unsigned tid = threadIdx.x;
    const unsigned lane = L > 1 ? tid / tile : 0u;  // op lane of this thread
    const unsigned ltid = L > 1 ? tid % tile : tid;
    const unsigned pl = ltid / G;  // pattern within the tile
    const unsigned g = ltid % G;   // component group of this thread
    const unsigned k0 = g * KT;    // its first component
    const unsigned p = tile_idx * tile + pl;
    const size_t ppad = a.ppad;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + Lay.bars);
    unsigned char *ring = smem + Lay.ring;
    V *slots = reinterpret_cast<V *>(smem + Lay.slots);
    S *slot_sc = reinterpret_cast<S *>(smem + Lay.slot_sc);
    // STAGED: every leaf's row is staged once per tile and records travel
    // alone (stage stride L records).  Else each stage carries its op's
    // leaf rows (stage stride Lay.stage).
    const size_t sstride = STAGED ? (size_t)a.rstride * L : Lay.stage;
    uint8_t *masks = smem + Lay.masks;
    const unsigned R = ring_depth;
    const unsigned nsteps = a.nops / L;  // the host pads nops to a multiple

    if (STAGED) {
        pdl_wait();  // the records hold the P kernel's matrices
        // Start streaming the job's first R steps of op records.
        if (tid == 0) {
            fence_proxy_async();
            for (unsigned o = 0; o < R && o < nsteps; ++o) {
                mbar_expect_tx(&bars[o], (uint32_t)sstride);
                bulk_g2s(ring + (size_t)o * sstride, a.rec + (size_t)o * sstride,
                         (uint32_t)sstride, &bars[o]);
            }
        }
        // Stage this tile's leaf masks with 16-byte loads.
        const unsigned chunks = tile / 16;
        for (unsigned i = tid; i < a.nleaf * chunks; i += nthr) {
            const unsigned l = i / chunks, c = i % chunks;
            const uint4 *src =
                reinterpret_cast<const uint4 *>(a.leaves[l] + (size_t)tile_idx * tile) + c;
            reinterpret_cast<uint4 *>(masks + (size_t)l * tile)[c] = __ldg(src);
        }
        __syncthreads();
    } else {
        pdl_wait();
        // Start streaming the job's first R stages (records and leaf rows).
        if (tid == 0)
            for (unsigned o = 0; o < R && o < a.nops; ++o) {
                const uint8_t *rows0[kLeafPre];
                read_rows(a, o, rows0);
                issue_stage(a, o, ring + (size_t)o * sstride, &bars[o], tile_idx, tile, rows0);
            }
    }

    T acc[KT * 4];
    S lns = S(0);
    // The last result this thread computed (its parent buffer and scaler;
    // the values are acc).  A child of the next op that is that buffer --
    // in a post-order, the next op is often the parent -- is taken from
    // registers instead of being read back: the same values, since the
    // stored FP32 row is acc itself.
    const void *prev_data = nullptr;
    S prev_lns = S(0);
    const uint32_t spin = g_spin_limit;
    for (unsigned o = 0, stage = 0; o < nsteps;
         ++o, stage = (stage + 1 == R) ? 0u : stage + 1) {
        // Streaming: thread 0 reads op o + R's leaf-row pointers now; it
        // issues that stage after this op, when the loads have long arrived.
        const uint8_t *pre[kLeafPre] = {nullptr, nullptr, nullptr, nullptr};
        if (!STAGED && tid == 0 && o + R < nsteps) read_rows(a, o + R, pre);
        // Every thread waits for the op's record itself (one block barrier
        // per op, the hand-off below); a warp computes only if all its
        // threads saw the record arrive.
        const bool ok =
            __all_sync(0xffffffffu, mbar_wait_bounded(&bars[stage], (phase >> stage) & 1u,
                                                      spin));
        phase ^= 1u << stage;
        void *ydata = nullptr, *yscaler = nullptr;
        int yslot = -1;
        bool yhbm = false;
        uint32_t nbytes = (uint32_t)sstride;
        unsigned nchild = 0;
        T sc = T(0);  // plain form: max over child messages
        if (ok) {
        const unsigned char *rec = ring + (size_t)stage * sstride + (size_t)lane * a.rstride;
        const uint8_t *lrow = rec + a.rstride;  // this op's leaf rows
        unsigned nlk = 0;  // leaf children of this op seen so far
        const RecHead *hd = reinterpret_cast<const RecHead *>(rec);
        const RecChild *kids = reinterpret_cast<const RecChild *>(rec + sizeof(RecHead));
        nchild = hd->nchild;
        lns = S(0);
        // A child's inputs: its state rows (internal) with its scaler, or
        // its leaf's state mask.  Loading them is split from computing the
        // message so that an op with two children issues both children's
        // loads before it waits on either.
        struct In {
            T x[KT * 4];
            S l;
            unsigned m;
        };
        auto load_in = [&](const RecChild &ch, In &in) {
            if (ch.src == SRC_LEAF) {
                in.m = STAGED ? masks[(size_t)ch.idx * tile + pl]
                              : lrow[(size_t)(nlk++) * tile + pl];
                return;
            }
            in.m = 0u;
            const bool in_slot = (ch.src == SRC_SLOT);
            const V *xs = in_slot ? slots + ((size_t)ch.idx * KA + k0) * U * tile + pl
                                  : static_cast<const V *>(ch.data) + (size_t)k0 * U * ppad + p;
            const size_t stride = in_slot ? tile : ppad;
#pragma unroll
            for (int k = 0; k < KT; ++k) load4<T>(xs + (size_t)k * U * stride, stride, in.x + k * 4);
            in.l = in_slot ? slot_sc[(size_t)ch.idx * tile + pl]
                           : static_cast<const S *>(ch.scaler)[p];
        };
        auto message = [&](const RecChild &ch, const In &in, T *msg) {
            const T *area = reinterpret_cast<const T *>(rec + ch.off);
            const V *P = reinterpret_cast<const V *>(area + (size_t)k0 * 16);
            const unsigned m = in.m;
            if (sizeof(T) == 4 && ch.src == SRC_LEAF) {
                // FP32 leaves: the message of mask m from the record's table.
                const float4 *t = reinterpret_cast<const float4 *>(area) + (size_t)k0 * 16 + m;
#pragma unroll
                for (int k = 0; k < KT; ++k) {
                    const float4 v = t[k * 16];
                    msg[k * 4 + 0] = (T)v.x;
                    msg[k * 4 + 1] = (T)v.y;
                    msg[k * 4 + 2] = (T)v.z;
                    msg[k * 4 + 3] = (T)v.w;
                }
            } else if (sizeof(T) == 8 && ch.src == SRC_LEAF) {
                // FP64 leaves: table lookup (no FP64 arithmetic).
                const double2 *t = reinterpret_cast<const double2 *>(
                    a.ltab + (((size_t)ch.tab * 16 + m) * KA + k0) * 4);
#pragma unroll
                for (int q = 0; q < KT * 2; ++q) {
                    const double2 v = __ldg(t + q);
                    msg[2 * q] = (T)v.x;
                    msg[2 * q + 1] = (T)v.y;
                }
            } else {
#pragma unroll
                for (int k = 0; k < KT; ++k) {
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        T r[4];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            T tmp[4 / U];
                            unpack(P[(k * 16 + i * 4) / (4 / U) + u], tmp);
#pragma unroll
                            for (int q = 0; q < 4 / U; ++q) r[u * (4 / U) + q] = tmp[q];
                        }
                        const T *x = in.x + k * 4;
                        T v = r[0] * x[0];
                        v = fma(r[1], x[1], v);
                        v = fma(r[2], x[2], v);
                        v = fma(r[3], x[3], v);
                        msg[k * 4 + i] = v;
                    }
                }
            }
        };
        // Fold child ci's message into the op: product of messages, sum of
        // scalers in child order; the plain form's scaler is the max over
        // every child message (CxLik.c:390-403).
        auto fold = [&](unsigned ci, const RecChild &ch, const In &in, const T *msg) {
            if (ch.src != SRC_LEAF) lns = lns + in.l;
            if (ci == 0) {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) acc[q] = msg[q];
            } else {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) acc[q] *= msg[q];
            }
            if constexpr (sizeof(T) == 8) sc = max_nonneg(sc, tree_max_nonneg<KT * 4>(msg));
        };
        // A two-child FP32 op whose kind the host set runs straight-line
        // code for its kind (the general path below gives the same bits).
        uint32_t kind = OPK_GENERIC;
        if constexpr (sizeof(T) == 4 && G == 1 && L == 1) {
            const uint32_t fl = hd->flags;
            kind = (fl >> kOpKindShift) & 7u;
            // A walk that starts inside a plan (one launch per node) holds
            // no previous result: its first op runs the general path, which
            // reads that child from where its record says.
            if ((kind == OPK_FL || kind == OPK_FI) && o == 0) kind = OPK_GENERIC;
            if (kind != OPK_GENERIC) {
                float(&acc1)[1][KT * 4] = reinterpret_cast<float(&)[1][KT * 4]>(acc);
                int l1[1] = {prev_lns};
                const unsigned pl1[1] = {pl}, p1[1] = {p};
                op2_kind<KT, STAGED, 1>(kind, rec, kids, (fl & kOpKindA) ? 1u : 0u, acc1, l1,
                                        masks, lrow, slots, slot_sc, tile, pl1, p1, ppad);
                lns = l1[0];
            }
        }
        // (The FP64 form keeps the loop: both children's rows in registers
        // at once cost it occupancy, and it is bound by the FP64 pipe.)
        if (kind != OPK_GENERIC) {
        } else if (sizeof(T) == 4 && !(G == 1 && L == 1) && nchild == 2) {
            const RecChild c0 = kids[0], c1 = kids[1];
            In in0, in1;
            const bool f0 = L == 1 && prev_data != nullptr && c0.src != SRC_LEAF &&
                            c0.data == prev_data;
            const bool f1 = L == 1 && prev_data != nullptr && c1.src != SRC_LEAF &&
                            c1.data == prev_data;
            if (f0) {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) in0.x[q] = acc[q];
                in0.l = prev_lns;
                in0.m = 0u;
            } else {
                load_in(c0, in0);
            }
            if (f1) {
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) in1.x[q] = acc[q];
                in1.l = prev_lns;
                in1.m = 0u;
            } else {
                load_in(c1, in1);
            }
            T msg[KT * 4];
            message(c0, in0, msg);
            fold(0, c0, in0, msg);
            message(c1, in1, msg);
            fold(1, c1, in1, msg);
        } else {
            for (unsigned ci = 0; ci < nchild; ++ci) {
                const RecChild ch = kids[ci];
                In in;
                load_in(ch, in);
                T msg[KT * 4];
                message(ch, in, msg);
                fold(ci, ch, in, msg);
            }
        }
        ydata = hd->data;
        yscaler = hd->scaler;
        yslot = hd->slot;
        yhbm = !(hd->flags & REC_NO_HBM);
        // Size of the record that refills this stage: only its own bytes
        // (records of internal children are a third of a leaf table's).
        nbytes = (L == 1 && hd->next_bytes != 0u && hd->next_bytes <= (uint32_t)sstride)
                     ? hd->next_bytes : (uint32_t)sstride;
        }  // ok
        // Every thread has read the stage: hand it to op o + R.  A record
        // wait that gave up in any warp ends the tile for all: thread 0
        // waits for the copies still in flight into the ring.  A one-warp
        // CTA needs only a warp barrier: every other shared row a thread
        // touches (stack slots, leaf masks) is its own pattern's.
        if (!cta_hand_off(ok, nthr)) {
            if (tid == 0) {
                atomicOr(a.err, 1u);
                drain_ring(bars, phase ^ (1u << stage), o, nsteps, R);
            }
            return false;
        }
        if (tid == 0 && o + R < nsteps) {
            if (STAGED) {
                fence_proxy_async();
                mbar_expect_tx(&bars[stage], nbytes);
                bulk_g2s(ring + (size_t)stage * sstride,
                         a.rec + (size_t)(o + R) * sstride, nbytes, &bars[stage]);
            } else {
                issue_stage(a, o + R, ring + (size_t)stage * sstride, &bars[stage], tile_idx,
                            tile, pre);
            }
        }
        // An empty lane of a step (no children) computes and stores nothing.
        if (L > 1 && nchild == 0) continue;
        if (sizeof(T) == 8) {
            if constexpr (sizeof(T) == 8) sc = group_max_nonneg<G>(sc);
            // Reference rescale: divide by the scaler unless it is 1, add
            // its log (a zero scaler gives NaN rows and a -inf site, as in
            // the reference).
            if (sc != T(1)) {
                const T r = T(1) / sc;
#pragma unroll
                for (int q = 0; q < KT * 4; ++q) acc[q] *= r;
            }
            lns = lns + (S)log((double)sc);
        } else {
            T mx = fmax(T(0), tree_max<KT * 4>(acc));
            mx = group_max<G>(mx);
            // Rescale only when the largest entry fell below 2^-16 (or the
            // op has more than two children): every entry is at most 1, a
            // binary op's result then keeps its largest entry far above the
            // FP32 normal range's floor, and scaling by a power of two is
            // exact, so each rescale that is skipped changes no mantissa.
            if (mx > T(0) && mx <= (T)3.0e38 && (nchild > 2 || mx < (T)1.52587890625e-05f)) {
                int e;
                frexpf((float)mx, &e);
                const int n = -e;
                if (n >= -126 && n <= 127) {
                    const float s1 = pow2f(n);
#pragma unroll
                    for (int q = 0; q < KT * 4; ++q) acc[q] *= (T)s1;
                } else {
                    const int n1 = n / 2, n2 = n - n1;
                    const float s1 = pow2f(n1), s2 = pow2f(n2);
#pragma unroll
                    for (int q = 0; q < KT * 4; ++q) acc[q] = (acc[q] * (T)s1) * (T)s2;
                }
                lns = lns + (S)e;
            }
        }
        if (yhbm) {
            V *y = static_cast<V *>(ydata) + (size_t)k0 * U * ppad + p;
#pragma unroll
            for (int k = 0; k < KT; ++k)
                store4<T>(y + (size_t)k * U * ppad, ppad, acc + k * 4);
            if (g == 0) static_cast<S *>(yscaler)[p] = lns;
        }
        if (yslot >= 0) {
            V *ys = slots + ((size_t)yslot * KA + k0) * U * tile + pl;
#pragma unroll
            for (int k = 0; k < KT; ++k) store4<T>(ys + (size_t)k * U * tile, tile, acc + k * 4);
            if (g == 0) slot_sc[(size_t)yslot * tile + pl] = lns;
        }
        prev_data = ydata;
        prev_lns = lns;
    }

    if (a.no_root) {
        __syncthreads();
        return true;
    }
    // Root aggregation (CxLik.c:598-632): L = sum_k sum_i pn[k][i] root.
    if (!a.root_last) {
        const V *r = static_cast<const V *>(a.root) + (size_t)k0 * U * ppad + p;
#pragma unroll
        for (int k = 0; k < KT; ++k) load4<T>(r + (size_t)k * U * ppad, ppad, acc + k * 4);
        lns = static_cast<const S *>(a.rootsc)[p];
    }
    // Lsum = sum over components and states in one sequential order; every
    // lane of the group gathers the others' entries and sums them all.
    double Lsum = 0.0;
    const unsigned lead = (tid & 31u) - g;
#pragma unroll
    for (int gg = 0; gg < G; ++gg) {
#pragma unroll
        for (int q = 0; q < KT * 4; ++q) {
            const T x = G > 1 ? __shfl_sync(0xffffffffu, acc[q], lead + gg) : acc[q];
            Lsum = fma(__ldg(a.pn + gg * KT * 4 + q), (double)x, Lsum);
        }
    }
    double v = 0.0;
    bool ninf = false;
    if (g == 0 && lane == 0 && p < a.npat) {
        const double lsc = (sizeof(T) == 8) ? (double)lns
                                           : (double)lns * 0.69314718055994530942;
        v = (log(Lsum) + lsc) * (double)a.freqs[p];
        if (isnan(v)) v = -INFINITY;
        if (a.site) a.site[p] = v;
        if (isinf(v)) {
            ninf = (v < 0.0);
            v = 0.0;
        }
    }
    if (G > 1) {
        // Pattern pl's value moves to thread pl, so the tile reduces in the
        // one-thread-per-pattern order (the extra threads add exact zeros).
        __shared__ double s_v[kBlock];
        __shared__ unsigned char s_inf[kBlock];
        if (g == 0) {
            s_v[pl] = v;
            s_inf[pl] = ninf;
        }
        __syncthreads();
        v = tid < tile ? s_v[tid] : 0.0;
        ninf = tid < tile ? s_inf[tid] != 0 : false;
    }
    reduce_sites(a, tile_idx, v, ninf);
    return true;
}

// The FP32 walker with two patterns per thread (one thread per pattern
// pair, components not split): thread t owns patterns t and t + blockDim
// of the tile, so loads stay coalesced, and every P row, record field and
// loop step serves both.  The arithmetic of each pattern is that of
// walk_tile<float, K, 1, STAGED>, and the tile reduction runs in its order,
// so the bits are the same.
template <int K, bool STAGED>
__device__ bool walk_tile2(const PlanArgs &a, unsigned tile_idx, const SmemLayout &Lay,
                           unsigned ring_depth, uint32_t &phase) {
    typedef float T;
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned nthr = blockDim.x;
    const unsigned tile = 2 * nthr;
    const unsigned tid = threadIdx.x;
    const unsigned pl[2] = {tid, tid + nthr};
    const unsigned p[2] = {tile_idx * tile + tid, tile_idx * tile + tid + nthr};
    const size_t ppad = a.ppad;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + Lay.bars);
    unsigned char *ring = smem + Lay.ring;
    float4 *slots = reinterpret_cast<float4 *>(smem + Lay.slots);
    int *slot_sc = reinterpret_cast<int *>(smem + Lay.slot_sc);
    const size_t sstride = STAGED ? (size_t)a.rstride : Lay.stage;
    uint8_t *masks = smem + Lay.masks;
    const unsigned R = ring_depth;

    if (STAGED) {
        pdl_wait();
        if (tid == 0) {
            fence_proxy_async();
            for (unsigned o = 0; o < R && o < a.nops; ++o) {
                mbar_expect_tx(&bars[o], a.rstride);
                bulk_g2s(ring + (size_t)o * a.rstride, a.rec + (size_t)o * a.rstride,
                         a.rstride, &bars[o]);
            }
        }
        const unsigned chunks = tile / 16;
        for (unsigned i = tid; i < a.nleaf * chunks; i += nthr) {
            const unsigned l = i / chunks, c = i % chunks;
            const uint4 *src =
                reinterpret_cast<const uint4 *>(a.leaves[l] + (size_t)tile_idx * tile) + c;
            reinterpret_cast<uint4 *>(masks + (size_t)l * tile)[c] = __ldg(src);
        }
        __syncthreads();
    } else {
        pdl_wait();
        if (tid == 0)
            for (unsigned o = 0; o < R && o < a.nops; ++o) {
                const uint8_t *rows0[kLeafPre];
                read_rows(a, o, rows0);
                issue_stage(a, o, ring + (size_t)o * sstride, &bars[o], tile_idx, tile, rows0);
            }
    }

    T acc[2][K * 4];
    int lns[2] = {0, 0};
    const uint32_t spin = g_spin_limit;
    for (unsigned o = 0, stage = 0; o < a.nops;
         ++o, stage = (stage + 1 == R) ? 0u : stage + 1) {
        const uint8_t *pre[kLeafPre] = {nullptr, nullptr, nullptr, nullptr};
        if (!STAGED && tid == 0 && o + R < a.nops) read_rows(a, o + R, pre);
        // Every thread waits for the record (walk_tile's hand-off).
        const bool ok =
            __all_sync(0xffffffffu, mbar_wait_bounded(&bars[stage], (phase >> stage) & 1u,
                                                      spin));
        phase ^= 1u << stage;
        void *ydata = nullptr, *yscaler = nullptr;
        int yslot = -1;
        bool yhbm = false;
        unsigned nchild = 0;
        uint32_t nbytes = (uint32_t)sstride;
        if (ok) {
        const unsigned char *rec = ring + (size_t)stage * sstride;
        const uint8_t *lrow = rec + a.rstride;
        unsigned nlk = 0;
        const RecHead *hd = reinterpret_cast<const RecHead *>(rec);
        const RecChild *kids = reinterpret_cast<const RecChild *>(rec + sizeof(RecHead));
        nchild = hd->nchild;
        const uint32_t fl = hd->flags;
        uint32_t kind = (fl >> kOpKindShift) & 7u;
        if ((kind == OPK_FL || kind == OPK_FI) && o == 0) kind = OPK_GENERIC;
        if (kind != OPK_GENERIC) {
            op2_kind<K, STAGED, 2>(kind, rec, kids, (fl & kOpKindA) ? 1u : 0u, acc, lns, masks,
                                   lrow, slots, slot_sc, tile, pl, p, ppad);
        } else {
        lns[0] = lns[1] = 0;
        for (unsigned ci = 0; ci < nchild; ++ci) {
            const RecChild ch = kids[ci];
            const float *area = reinterpret_cast<const float *>(rec + ch.off);
            T msg[2][K * 4];
            if (ch.src == SRC_LEAF) {
                unsigned m[2];
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    m[h] = STAGED ? masks[(size_t)ch.idx * tile + pl[h]]
                                  : lrow[(size_t)nlk * tile + pl[h]];
                if (!STAGED) ++nlk;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float4 *t = reinterpret_cast<const float4 *>(area) + m[h];
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        const float4 v = t[k * 16];
                        msg[h][k * 4 + 0] = v.x;
                        msg[h][k * 4 + 1] = v.y;
                        msg[h][k * 4 + 2] = v.z;
                        msg[h][k * 4 + 3] = v.w;
                    }
                }
            } else {
                const bool in_slot = (ch.src == SRC_SLOT);
                const float4 *P = reinterpret_cast<const float4 *>(area);
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    float x[2][4];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const float4 v =
                            in_slot ? slots[((size_t)ch.idx * K + k) * tile + pl[h]]
                                    : static_cast<const float4 *>(ch.data)[(size_t)k * ppad + p[h]];
                        unpack(v, x[h]);
                    }
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        float r[4];
                        unpack(P[k * 4 + i], r);
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            float v = r[0] * x[h][0];
                            v = fmaf(r[1], x[h][1], v);
                            v = fmaf(r[2], x[h][2], v);
                            v = fmaf(r[3], x[h][3], v);
                            msg[h][k * 4 + i] = v;
                        }
                    }
                }
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    lns[h] += in_slot ? slot_sc[(size_t)ch.idx * tile + pl[h]]
                                      : static_cast<const int *>(ch.scaler)[p[h]];
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (ci == 0) {
#pragma unroll
                    for (int q = 0; q < K * 4; ++q) acc[h][q] = msg[h][q];
                } else {
#pragma unroll
                    for (int q = 0; q < K * 4; ++q) acc[h][q] *= msg[h][q];
                }
            }
        }
        }  // generic
        ydata = hd->data;
        yscaler = hd->scaler;
        yslot = hd->slot;
        yhbm = !(fl & REC_NO_HBM);
        nbytes = (hd->next_bytes != 0u && hd->next_bytes <= (uint32_t)sstride)
                     ? hd->next_bytes : (uint32_t)sstride;
        }  // ok
        if (!cta_hand_off(ok, nthr)) {
            if (tid == 0) {
                atomicOr(a.err, 1u);
                drain_ring(bars, phase ^ (1u << stage), o, a.nops, R);
            }
            return false;
        }
        if (tid == 0 && o + R < a.nops) {
            if (STAGED) {
                fence_proxy_async();
                mbar_expect_tx(&bars[stage], nbytes);
                bulk_g2s(ring + (size_t)stage * a.rstride,
                         a.rec + (size_t)(o + R) * a.rstride, nbytes, &bars[stage]);
            } else {
                issue_stage(a, o + R, ring + (size_t)stage * sstride, &bars[stage], tile_idx,
                            tile, pre);
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            T mx = T(0);
#pragma unroll
            for (int q = 0; q < K * 4; ++q) mx = fmax(mx, acc[h][q]);
            // The rescale rule of walk_tile (same bits).
            if (mx > T(0) && mx <= (T)3.0e38 && (nchild > 2 || mx < 1.52587890625e-05f)) {
                int e;
                frexpf(mx, &e);
                const int n = -e;
                if (n >= -126 && n <= 127) {
                    const float s1 = pow2f(n);
#pragma unroll
                    for (int q = 0; q < K * 4; ++q) acc[h][q] *= s1;
                } else {
                    const int n1 = n / 2, n2 = n - n1;
                    const float s1 = pow2f(n1), s2 = pow2f(n2);
#pragma unroll
                    for (int q = 0; q < K * 4; ++q) acc[h][q] = (acc[h][q] * s1) * s2;
                }
                lns[h] += e;
            }
            if (yhbm) {
                float4 *y = static_cast<float4 *>(ydata) + p[h];
#pragma unroll
                for (int k = 0; k < K; ++k) y[(size_t)k * ppad] = pack4(acc[h] + k * 4);
                static_cast<int *>(yscaler)[p[h]] = lns[h];
            }
            if (yslot >= 0) {
                float4 *ys = slots + (size_t)yslot * K * tile + pl[h];
#pragma unroll
                for (int k = 0; k < K; ++k) ys[(size_t)k * tile] = pack4(acc[h] + k * 4);
                slot_sc[(size_t)yslot * tile + pl[h]] = lns[h];
            }
        }
    }

    if (a.no_root) {
        __syncthreads();
        return true;
    }
    double v[2] = {0.0, 0.0};
    bool ninf[2] = {false, false};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (!a.root_last) {
            const float4 *r = static_cast<const float4 *>(a.root) + p[h];
#pragma unroll
            for (int k = 0; k < K; ++k) unpack(r[(size_t)k * ppad], acc[h] + k * 4);
            lns[h] = static_cast<const int *>(a.rootsc)[p[h]];
        }
        double L = 0.0;
#pragma unroll
        for (int q = 0; q < K * 4; ++q) L = fma(__ldg(a.pn + q), (double)acc[h][q], L);
        if (p[h] < a.npat) {
            v[h] = (log(L) + (double)lns[h] * 0.69314718055994530942) * (double)a.freqs[p[h]];
            if (isnan(v[h])) v[h] = -INFINITY;
            if (a.site) a.site[p[h]] = v[h];
            if (isinf(v[h])) {
                ninf[h] = (v[h] < 0.0);
                v[h] = 0.0;
            }
        }
    }
    reduce_sites_n<2>(a, tile_idx, v, ninf);
    return true;
}

// A batched job's arguments, copied into shared memory when a CTA's next
// item belongs to another job: read through a pointer into global memory,
// every field would be reloaded after each store the walker makes.  The
// previous item ended with a block barrier, so no thread still reads the
// old copy.
static_assert(sizeof(PlanArgs) % 8 == 0, "PlanArgs is copied in 8-byte words");
__device__ __forceinline__ void load_job(PlanArgs &dst, const PlanArgs *src) {
    const unsigned long long *s = reinterpret_cast<const unsigned long long *>(src);
    unsigned long long *d = reinterpret_cast<unsigned long long *>(&dst);
    for (unsigned i = threadIdx.x; i < sizeof(PlanArgs) / 8; i += blockDim.x) d[i] = s[i];
    __syncthreads();
}

__device__ __forceinline__ void init_ring(const SmemLayout &Lay, unsigned R) {
    extern __shared__ __align__(128) unsigned char smem[];
    if (threadIdx.x == 0) {
        uint64_t *bars = reinterpret_cast<uint64_t *>(smem + Lay.bars);
        for (unsigned r = 0; r < R; ++r) mbar_init(&bars[r], 1);
        fence_mbar_init();
    }
    __syncthreads();
}

// Register cap of the FP32 walkers with up to five components a thread:
// 128.  A 70,000-pattern tree is 1,100 tiles of 64 patterns, and eight
// 64-thread CTAs per SM (one wave on 152 SMs) need registers <= 128; above,
// a second wave doubles the tail.  Wider shapes keep the compiler's choice.
template <typename T, int KT>
constexpr int walker_min_blocks() {
    return (sizeof(T) == 4 && KT <= 5) ? 2 : 1;
}

// One plan: one CTA per tile.
template <typename T, int KT, int G, bool STAGED>
__global__ void __launch_bounds__(kMaxThreads, walker_min_blocks<T, KT>())
    walk_kernel(PlanArgs a) {
    const SmemLayout Lay = smem_layout(sizeof(T) == 4 ? CXG_FP32 : CXG_FP64, KT * G,
                                       blockDim.x / G, a.nslot, a.ring,
                                       a.rstride, a.lmax, a.nleaf);
    init_ring(Lay, a.ring);
    uint32_t phase = 0;
    walk_tile<T, KT, G, STAGED>(a, blockIdx.x, Lay, a.ring, phase);
}

// One plan with L = 2 op lanes (FP32, one thread per pattern, staged
// leaves): one CTA of NT = 2 x tile threads per tile, tile <= 64.  The
// bounds keep a 70,000-pattern tree (1,100 tiles of 64, 2,200 of 32) in one
// wave on 152 SMs: eight 128-thread CTAs per SM (64 registers) or fifteen
// 64-thread CTAs (68 registers).
template <int K, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) walk_kernel_lanes(PlanArgs a) {
    const SmemLayout Lay = smem_layout(CXG_FP32, K, blockDim.x / 2, a.nslot, a.ring,
                                       a.rstride * 2, 0, a.nleaf);
    init_ring(Lay, a.ring);
    uint32_t phase = 0;
    walk_tile<float, K, 1, true, 2>(a, blockIdx.x, Lay, a.ring, phase);
}

// Many jobs: a persistent grid claims (job, tile) items in the host's order
// (longest first).
template <typename T, int KT, int G, bool STAGED>
__global__ void __launch_bounds__(kMaxThreads, walker_min_blocks<T, KT>())
    walk_batch_kernel(BatchArgs b) {
    __shared__ unsigned s_item;
    __shared__ __align__(16) PlanArgs s_job;
    const SmemLayout Lay = smem_layout(sizeof(T) == 4 ? CXG_FP32 : CXG_FP64, KT * G,
                                       blockDim.x / G, b.max_nslot,
                                       b.ring, b.max_rstride, b.max_lmax,
                                       b.max_nleaf);
    init_ring(Lay, b.ring);
    uint32_t phase = 0;
    unsigned job = ~0u;
    for (unsigned n = 0;; ++n) {
        unsigned item;
        if (b.direct) {
            item = n == 0 ? blockIdx.x : b.nitems;
        } else {
            if (threadIdx.x == 0) s_item = atomicAdd(b.counter, 1u);
            __syncthreads();
            item = s_item;
            __syncthreads();
        }
        if (item >= b.nitems) break;
        const WalkItem it = b.items[item];
        if (it.job != job) {
            load_job(s_job, b.jobs + it.job);
            job = it.job;
        }
        if (!walk_tile<T, KT, G, STAGED>(s_job, it.tile, Lay, b.ring, phase)) break;
    }
}

// Two patterns per thread (FP32, one thread per pattern pair).
template <int K, bool STAGED>
__global__ void __launch_bounds__(kBlock) walk_kernel2(PlanArgs a) {
    const SmemLayout Lay = smem_layout(CXG_FP32, K, blockDim.x * 2, a.nslot, a.ring,
                                       a.rstride, a.lmax, a.nleaf);
    init_ring(Lay, a.ring);
    uint32_t phase = 0;
    walk_tile2<K, STAGED>(a, blockIdx.x, Lay, a.ring, phase);
}

template <int K, bool STAGED>
__global__ void __launch_bounds__(kBlock) walk_batch_kernel2(BatchArgs b) {
    __shared__ unsigned s_item;
    __shared__ __align__(16) PlanArgs s_job;
    unsigned job = ~0u;
    const SmemLayout Lay = smem_layout(CXG_FP32, K, blockDim.x * 2, b.max_nslot, b.ring,
                                       b.max_rstride, b.max_lmax, b.max_nleaf);
    init_ring(Lay, b.ring);
    uint32_t phase = 0;
    for (unsigned n = 0;; ++n) {
        unsigned item;
        if (b.direct) {
            item = n == 0 ? blockIdx.x : b.nitems;
        } else {
            if (threadIdx.x == 0) s_item = atomicAdd(b.counter, 1u);
            __syncthreads();
            item = s_item;
            __syncthreads();
        }
        if (item >= b.nitems) break;
        const WalkItem it = b.items[item];
        if (it.job != job) {
            load_job(s_job, b.jobs + it.job);
            job = it.job;
        }
        if (!walk_tile2<K, STAGED>(s_job, it.tile, Lay, b.ring, phase)) break;
    }
}

unsigned plan_blocks(unsigned ppad, unsigned tile) { return ppad / tile; }

template <typename Kern>
static cudaError_t ensure_smem(Kern k, size_t sm, size_t &optin) {
    // Raised on every new maximum, not only above 48 KiB: the default limit
    // counts static and dynamic shared memory together, so a dynamic size
    // just under 48 KiB plus the walker's static arrays would not launch.
    // Several host threads launch walkers (the server's workers): the
    // attribute only grows, under one lock.
    static std::mutex mu;
    std::lock_guard<std::mutex> g(mu);
    if (sm > optin) {
        cudaError_t e = cudaFuncSetAttribute(
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        optin = sm;
    }
    return cudaSuccess;
}

// Instantiated walker shapes (per-thread components KT, threads per
// pattern G): every kact with G = 1; the FP32 form also splits a pattern's
// components over 2 or 4 threads (walker_shape_ok).
#define CXG_SHAPES_G1(X) X(1, 1) X(2, 1) X(3, 1) X(4, 1) X(5, 1) X(6, 1) X(7, 1) X(8, 1)
#define CXG_SHAPES_GN(X) X(1, 2) X(2, 2) X(3, 2) X(4, 2) X(1, 4) X(2, 4)

template <typename T, int KT, int G, bool ST>
static cudaError_t walk_fn(size_t sm, void (**fn)(PlanArgs)) {
    static size_t optin = 0;
    *fn = walk_kernel<T, KT, G, ST>;
    return ensure_smem(walk_kernel<T, KT, G, ST>, sm, optin);
}
template <typename T, int KT, int G, bool ST>
static cudaError_t batch_fn(size_t sm, void (**fn)(BatchArgs)) {
    static size_t optin = 0;
    *fn = walk_batch_kernel<T, KT, G, ST>;
    return ensure_smem(walk_batch_kernel<T, KT, G, ST>, sm, optin);
}
template <int K, int NT, int MINB>
static cudaError_t lanes_fn(size_t sm, void (**fn)(PlanArgs)) {
    static size_t optin = 0;
    *fn = walk_kernel_lanes<K, NT, MINB>;
    return ensure_smem(walk_kernel_lanes<K, NT, MINB>, sm, optin);
}
template <int K, bool ST>
static cudaError_t walk2_fn(size_t sm, void (**fn)(PlanArgs)) {
    static size_t optin = 0;
    *fn = walk_kernel2<K, ST>;
    return ensure_smem(walk_kernel2<K, ST>, sm, optin);
}
template <int K, bool ST>
static cudaError_t batch2_fn(size_t sm, void (**fn)(BatchArgs)) {
    static size_t optin = 0;
    *fn = walk_batch_kernel2<K, ST>;
    return ensure_smem(walk_batch_kernel2<K, ST>, sm, optin);
}

// The two-patterns-per-thread walker for kact (FP32), with its dynamic
// shared memory limit raised to `sm` bytes.
template <typename Fn>
static cudaError_t pick_walker2(unsigned kact, bool staged, size_t sm, Fn *fn, bool batch) {
#define CXG_X2(K)                                                                       \
    if (kact == (K)) {                                                                  \
        if (batch)                                                                      \
            return staged ? batch2_fn<K, true>(sm, reinterpret_cast<void (**)(BatchArgs)>(fn)) \
                          : batch2_fn<K, false>(sm, reinterpret_cast<void (**)(BatchArgs)>(fn)); \
        return staged ? walk2_fn<K, true>(sm, reinterpret_cast<void (**)(PlanArgs)>(fn))       \
                      : walk2_fn<K, false>(sm, reinterpret_cast<void (**)(PlanArgs)>(fn));     \
    }
    CXG_X2(1) CXG_X2(2) CXG_X2(3) CXG_X2(4) CXG_X2(5)
#undef CXG_X2
    return cudaErrorInvalidValue;
}

// The walker for (kact, G, staged leaves or streamed), with its dynamic
// shared memory limit raised to `sm` bytes.
template <typename T, typename Fn>
static cudaError_t pick_walker(unsigned kact, unsigned G, bool staged, size_t sm, Fn *fn,
                               bool batch) {
#define CXG_X(KT, GG)                                                              \
    if (kact == (KT) * (GG) && G == (GG)) {                                        \
        if (batch)                                                                 \
            return staged ? batch_fn<T, KT, GG, true>(                             \
                                sm, reinterpret_cast<void (**)(BatchArgs)>(fn))    \
                          : batch_fn<T, KT, GG, false>(                            \
                                sm, reinterpret_cast<void (**)(BatchArgs)>(fn));   \
        return staged ? walk_fn<T, KT, GG, true>(                                  \
                            sm, reinterpret_cast<void (**)(PlanArgs)>(fn))         \
                      : walk_fn<T, KT, GG, false>(                                 \
                            sm, reinterpret_cast<void (**)(PlanArgs)>(fn));        \
    }
    CXG_SHAPES_G1(CXG_X)
    if constexpr (sizeof(T) == 4) {
        CXG_SHAPES_GN(CXG_X)
    }
#undef CXG_X
    return cudaErrorInvalidValue;
}

// The op-lane walker for kact (FP32), with its dynamic shared memory limit
// raised to `sm` bytes.
static cudaError_t pick_walker_lanes(unsigned kact, unsigned tile, size_t sm,
                                     void (**fn)(PlanArgs)) {
#define CXG_XL(K) \
    if (kact == (K))                                                      \
        return tile == 64 ? lanes_fn<K, 128, 8>(sm, fn) : lanes_fn<K, 64, 15>(sm, fn);
    CXG_XL(1) CXG_XL(2) CXG_XL(3) CXG_XL(4) CXG_XL(5)
#undef CXG_XL
    return cudaErrorInvalidValue;
}

template <typename T>
static cudaError_t launch_plan_t(int precision, const PlanArgs &a, unsigned lanes,
                                 bool pdl, cudaStream_t s) {
    const unsigned G = a.tpp ? a.tpp : 1, NP = a.ppt ? a.ppt : 1;
    const unsigned nb = plan_blocks(a.ppad, a.tile);
    const size_t sm = plan_smem_bytes(precision, a.kact, a.tile, a.nslot,
                                      a.ring, a.rstride * lanes, a.lmax, a.nleaf);
    void (*fn)(PlanArgs) = nullptr;
    cudaError_t e = lanes == 2 ? pick_walker_lanes(a.kact, a.tile, sm, &fn)
                    : NP == 2  ? pick_walker2(a.kact, a.lmax == 0, sm, &fn, false)
                               : pick_walker<T>(a.kact, G, a.lmax == 0, sm, &fn, false);
    if (e != cudaSuccess) return e;
    const unsigned nt = a.tile * G * lanes / NP;
    if (pdl) {
        // A dependent of the P kernel just before it on the stream.
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(nb);
        cfg.blockDim = dim3(nt);
        cfg.dynamicSmemBytes = sm;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, fn, a);
    }
    fn<<<nb, nt, sm, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_plan(int precision, const PlanArgs &a, cudaStream_t s, unsigned lanes,
                        bool pdl) {
    const unsigned G = a.tpp ? a.tpp : 1, NP = a.ppt ? a.ppt : 1;
    if (a.tile == 0 || a.tile > kBlock || a.tile % 32 || a.ppad % a.tile ||
        a.tile * G > kMaxThreads || a.tile / NP < 32 ||
        !walker_shape_ok(precision, a.kact, G, NP) ||
        a.ring == 0 || a.ring > 8 || a.rstride % 16 || a.rstride == 0 ||
        a.ntiles != a.ppad / a.tile)
        return cudaErrorInvalidValue;
    if (lanes != 1 && !(lanes == 2 && lanes_shape_ok(precision, a.kact, G, NP) &&
                        a.lmax == 0 && a.tile * lanes <= kLaneThreads &&
                        a.nops % lanes == 0))
        return cudaErrorInvalidValue;
    return precision == CXG_FP32 ? launch_plan_t<float>(precision, a, lanes, pdl, s)
                                 : launch_plan_t<double>(precision, a, lanes, pdl, s);
}

template <typename T>
static cudaError_t launch_batch_t(int precision, const BatchArgs &b,
                                  unsigned grid, cudaStream_t s) {
    const unsigned G = b.tpp ? b.tpp : 1, NP = b.ppt ? b.ppt : 1;
    const size_t sm = plan_smem_bytes(precision, b.kact, b.tile, b.max_nslot,
                                      b.ring, b.max_rstride, b.max_lmax,
                                      b.max_nleaf);
    void (*fn)(BatchArgs) = nullptr;
    cudaError_t e = NP == 2 ? pick_walker2(b.kact, b.max_lmax == 0, sm, &fn, true)
                            : pick_walker<T>(b.kact, G, b.max_lmax == 0, sm, &fn, true);
    if (e != cudaSuccess) return e;
    fn<<<grid, b.tile * G / NP, sm, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch(int precision, const BatchArgs &b_in, unsigned grid,
                         cudaStream_t s) {
    // Items that fit one persistent grid get one CTA each: the hardware
    // spreads those CTAs over the SMs evenly, where persistent CTAs that
    // claim items first would crowd onto some SMs.
    BatchArgs b = b_in;
    if (b.nitems > 0 && b.nitems <= grid) {
        b.direct = 1;
        grid = b.nitems;
    }
    const unsigned G = b.tpp ? b.tpp : 1, NP = b.ppt ? b.ppt : 1;
    if (b.tile == 0 || b.tile > kBlock || b.tile % 32 || b.tile * G > kMaxThreads ||
        b.tile / NP < 32 || !walker_shape_ok(precision, b.kact, G, NP) || b.ring == 0 ||
        b.ring > 8 || b.max_rstride % 16 || b.max_rstride == 0 || grid == 0)
        return cudaErrorInvalidValue;
    return precision == CXG_FP32 ? launch_batch_t<float>(precision, b, grid, s)
                                 : launch_batch_t<double>(precision, b, grid, s);
}

template <typename T>
static int batch_occ_t(unsigned kact, unsigned tile, unsigned G, unsigned NP, bool staged,
                       size_t smem) {
    void (*fn)(BatchArgs) = nullptr;
    cudaError_t e = NP == 2 ? pick_walker2(kact, staged, smem, &fn, true)
                            : pick_walker<T>(kact, G, staged, smem, &fn, true);
    int n = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, (int)(tile * G / NP), smem);
    return e == cudaSuccess ? n : 0;
}

int batch_ctas_per_sm(int precision, unsigned kact, unsigned tile, unsigned tpp,
                      unsigned ppt, bool staged, size_t smem) {
    const unsigned G = tpp ? tpp : 1, NP = ppt ? ppt : 1;
    if (!walker_shape_ok(precision, kact, G, NP) || tile * G > kMaxThreads || tile / NP < 32)
        return 0;
    return precision == CXG_FP32 ? batch_occ_t<float>(kact, tile, G, NP, staged, smem)
                                 : batch_occ_t<double>(kact, tile, G, NP, staged, smem);
}

__global__ void qdecomp_kernel(const double *rtri, const double *pi,
                               double *out) {
    if (blockIdx.x == 0 && threadIdx.x < 4) qdecomp4_warp(rtri, pi, out, 0);
}

cudaError_t launch_qdecomp(const double *rtri, const double *pi, double *out,
                           cudaStream_t s) {
    qdecomp_kernel<<<1, 32, 0, s>>>(rtri, pi, out);
    return cudaGetLastError();
}

}  // namespace cxg
