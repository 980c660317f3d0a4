// Pattern compression on the device: the sorted unique columns of an
// alignment with summed frequencies, as Alignment.compact computes them
// (pkg/Crux/CTMatrix.pyx:949-1031, after canonize :856-887): characters are
// canonicalised, columns are ordered bytewise (memcmp order of the
// canonical codes) and identical columns merge, adding their frequencies.
// The leaf-tip encoder writes the state masks the plan walker reads
// (Lik.pyx:1466-1475: the charType's value table, 0 -> "any").
//
//   0. compact_used: which canonical codes occur (a 256-entry flag table,
//      read back); the rank of a character is the position of its
//      canonical code among those, in byte order, so rank order is byte
//      order and a rank fits `bits` bits (3 for ACGT, N and gaps).
//   1. compact_transpose: rows [ntaxa][nsites] -> column-major ranks
//      [nsites][W] through a shared-memory tile.
//   2. LSD sort: for each chunk of `cpk` characters, last chunk first, pack
//      the chunk of every column (in the current order) into a 64-bit key,
//      first character most significant, and stable-radix-sort (key, column
//      index) pairs (cub::DeviceRadixSort, a CUDA toolkit primitive).
//   3. compact_flags: a column starts a pattern unless it equals the one
//      before it (16-byte compares); a scan numbers the patterns.
//   4. compact_scatter / compact_emit: the first column of each pattern
//      represents it, frequencies add (integer atomics: exact), and the
//      canonical rows and state masks of the patterns are written.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "cxg_internal.h"

namespace cxg {
namespace {

constexpr unsigned kTT = 32;  // transpose tile (taxa x sites)

// used[c] = 1 for every canonical code c that occurs.
__global__ void compact_used(const uint8_t *rows, size_t n, const uint8_t *canon,
                             uint32_t *used) {
    __shared__ uint32_t u[256];
    for (unsigned i = threadIdx.x; i < 256; i += blockDim.x) u[i] = 0;
    __syncthreads();
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        u[canon[rows[i]]] = 1;
    __syncthreads();
    for (unsigned i = threadIdx.x; i < 256; i += blockDim.x)
        if (u[i]) used[i] = 1;
}

// cols[s][t] = rank[rows[t][s]] for t < ntaxa, 0 (the smallest rank) for
// the padding taxa up to W.
__global__ void compact_transpose(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                                  unsigned W, const uint8_t *rank, uint8_t *cols) {
    __shared__ uint8_t t[kTT][kTT + 4];
    const unsigned s0 = blockIdx.x * kTT, t0 = blockIdx.y * kTT;
    for (unsigned i = threadIdx.y; i < kTT; i += blockDim.y) {
        const unsigned tx = t0 + i, sx = s0 + threadIdx.x;
        t[i][threadIdx.x] =
            (tx < ntaxa && sx < nsites) ? rank[rows[(size_t)tx * nsites + sx]] : 0;
    }
    __syncthreads();
    for (unsigned i = threadIdx.y; i < kTT; i += blockDim.y) {
        const unsigned sx = s0 + i, tx = t0 + threadIdx.x;
        if (sx < nsites && tx < W) cols[(size_t)sx * W + tx] = t[threadIdx.x][i];
    }
}

// key[i] = characters [c*cpk, c*cpk + cpk) of column idx[i], `bits` bits
// each, the first one most significant (beyond W: rank 0).
__global__ void compact_keys(const uint8_t *cols, unsigned W, const uint32_t *idx,
                             unsigned n, unsigned c, unsigned bits, unsigned cpk,
                             unsigned long long *key) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t *col = cols + (size_t)idx[i] * W;
    unsigned long long k = 0;
    for (unsigned j = 0; j < cpk; ++j) {
        const unsigned t = c * cpk + j;
        k = (k << bits) | (t < W ? col[t] : 0u);
    }
    key[i] = k;
}

// flag[i] = 1 if column idx[i] differs from column idx[i - 1] (or i == 0).
__global__ void compact_flags(const uint8_t *cols, unsigned W, const uint32_t *idx,
                              unsigned n, uint32_t *flag) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i == 0) {
        flag[0] = 1;
        return;
    }
    const uint4 *a = reinterpret_cast<const uint4 *>(cols + (size_t)idx[i] * W);
    const uint4 *b = reinterpret_cast<const uint4 *>(cols + (size_t)idx[i - 1] * W);
    uint32_t diff = 0;
    for (unsigned q = 0; q < W / 16 && !diff; ++q) {
        const uint4 x = a[q], y = b[q];
        diff = (x.x != y.x) | (x.y != y.y) | (x.z != y.z) | (x.w != y.w);
    }
    flag[i] = diff;
}

// Pattern g = gid[i] - 1 (gid: inclusive scan of the flags): its first
// column represents it; frequencies add.
__global__ void compact_scatter(const uint32_t *idx, const uint32_t *flag,
                                const uint32_t *gid, unsigned n, const uint32_t *freq_in,
                                uint32_t *rep, uint32_t *freq_out) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned g = gid[i] - 1;
    if (flag[i]) rep[g] = idx[i];
    atomicAdd(&freq_out[g], freq_in ? freq_in[idx[i]] : 1u);
}

// rows_out[t][g] = canon[rows[t][rep[g]]]; masks[t][g] = val of that code
// (0 -> any_mask); pad patterns g in [npat, mpad) of the masks get any_mask.
__global__ void compact_emit(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                             const uint32_t *rep, const uint32_t *npat_dev,
                             const uint8_t *canon, const uint8_t *val, uint8_t any_mask,
                             uint8_t *rows_out, unsigned rstride, uint8_t *masks,
                             unsigned mstride) {
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned t = blockIdx.y;
    const unsigned npat = *npat_dev;
    if (t >= ntaxa) return;
    if (g < npat) {
        const uint8_t c = canon[rows[(size_t)t * nsites + rep[g]]];
        if (rows_out) rows_out[(size_t)t * rstride + g] = c;
        if (masks) {
            const uint8_t v = val[c] & 15;
            masks[(size_t)t * mstride + g] = v ? v : any_mask;
        }
    } else if (masks && g < mstride) {
        masks[(size_t)t * mstride + g] = any_mask;
    }
}

size_t al256c(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// Rank table over the canonical codes that occur (used[code] != 0), in
// byte order, and the bits a rank needs.
static void compact_tables(const uint8_t *canon, const uint32_t *used, uint8_t *rank,
                           unsigned *bits) {
    unsigned r = 0;
    uint8_t code_rank[256] = {};
    for (int c = 0; c < 256; ++c)
        if (used[c]) code_rank[c] = (uint8_t)r++;
    for (int c = 0; c < 256; ++c) rank[c] = code_rank[canon[c]];
    unsigned b = 1;
    while ((1u << b) < r) ++b;
    *bits = b;
}

// Device compaction: inputs and outputs in device memory, on `s`.
// canon_host is the host copy of canon; canon and val are 256-entry device
// tables.  *npat_dev receives the pattern count.  `work` is scratch of
// compact_work_bytes(ntaxa, nsites) bytes.  Waits for the stream once (the
// codes in use decide the key width).
size_t compact_work_bytes(unsigned ntaxa, unsigned nsites) {
    const unsigned W = (ntaxa + 15) / 16 * 16;
    size_t cub_bytes = 0, scan_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, (const unsigned long long *)nullptr,
                                    (unsigned long long *)nullptr, (const uint32_t *)nullptr,
                                    (uint32_t *)nullptr, (int)nsites);
    cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, (const uint32_t *)nullptr,
                                  (uint32_t *)nullptr, (int)nsites);
    const size_t n = nsites;
    return 2048 + al256c(n * W) + 2 * al256c(n * 8) + 4 * al256c(n * 4) +
           al256c(cub_bytes > scan_bytes ? cub_bytes : scan_bytes);
}

int compact_device(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                   const uint32_t *freq_in, const uint8_t *canon_host, const uint8_t *canon,
                   const uint8_t *val, uint8_t any_mask, uint8_t *rows_out, unsigned rstride,
                   uint8_t *masks, unsigned mstride, uint32_t *freq_out, uint32_t *npat_dev,
                   void *work, size_t work_bytes, cudaStream_t s) {
    const unsigned W = (ntaxa + 15) / 16 * 16;
    const size_t n = nsites;
    if (compact_work_bytes(ntaxa, nsites) > work_bytes)
        return fail(CXG_EINVAL, "compaction: scratch too small");
    char *p = static_cast<char *>(work);
    auto take = [&](size_t b) {
        char *q = p;
        p += al256c(b);
        return q;
    };
    uint32_t *used = (uint32_t *)take(1024);
    uint8_t *rank = (uint8_t *)take(256);
    // The canonical codes in use decide the rank table and key width.
    CXG_CUDA(cudaMemsetAsync(used, 0, 1024, s));
    compact_used<<<304, 256, 0, s>>>(rows, (size_t)ntaxa * nsites, canon, used);
    CXG_CHECK_LAUNCH("compact_used");
    uint32_t used_h[256];
    CXG_CUDA(cudaMemcpyAsync(used_h, used, 1024, cudaMemcpyDeviceToHost, s));
    CXG_CUDA(cudaStreamSynchronize(s));
    uint8_t rank_h[256];
    unsigned bits = 8;
    compact_tables(canon_host, used_h, rank_h, &bits);
    CXG_CUDA(cudaMemcpyAsync(rank, rank_h, 256, cudaMemcpyHostToDevice, s));
    uint8_t *cols = (uint8_t *)take(n * W);
    unsigned long long *k0 = (unsigned long long *)take(n * 8);
    unsigned long long *k1 = (unsigned long long *)take(n * 8);
    uint32_t *i0 = (uint32_t *)take(n * 4);
    uint32_t *i1 = (uint32_t *)take(n * 4);
    uint32_t *flag = (uint32_t *)take(n * 4);
    uint32_t *gid = (uint32_t *)take(n * 4);
    size_t cub_bytes = work_bytes - (size_t)(p - static_cast<char *>(work));
    void *cub_tmp = p;

    dim3 tb(kTT, 8), tg((nsites + kTT - 1) / kTT, (W + kTT - 1) / kTT);
    compact_transpose<<<tg, tb, 0, s>>>(rows, ntaxa, nsites, W, rank, cols);
    CXG_CHECK_LAUNCH("compact_transpose");
    // Identity order, then one stable sort per key chunk, last chunk first.
    std::vector<uint32_t> iota(n);
    for (size_t i = 0; i < n; ++i) iota[i] = (uint32_t)i;
    CXG_CUDA(cudaMemcpyAsync(i0, iota.data(), n * 4, cudaMemcpyHostToDevice, s));
    const unsigned cpk = 64 / bits;
    const unsigned nchunks = (W + cpk - 1) / cpk;
    const unsigned nb = (unsigned)((n + 255) / 256);
    for (int c = (int)nchunks - 1; c >= 0; --c) {
        compact_keys<<<nb, 256, 0, s>>>(cols, W, i0, (unsigned)n, (unsigned)c, bits, cpk, k0);
        CXG_CHECK_LAUNCH("compact_keys");
        cudaError_t e = cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, k0, k1, i0, i1,
                                                        (int)n, 0, (int)(cpk * bits), s);
        if (e != cudaSuccess) return cuda_fail(e, "compaction radix sort");
        uint32_t *t = i0;
        i0 = i1;
        i1 = t;
    }
    compact_flags<<<nb, 256, 0, s>>>(cols, W, i0, (unsigned)n, flag);
    CXG_CHECK_LAUNCH("compact_flags");
    cudaError_t e = cub::DeviceScan::InclusiveSum(cub_tmp, cub_bytes, flag, gid, (int)n, s);
    if (e != cudaSuccess) return cuda_fail(e, "compaction scan");
    CXG_CUDA(cudaMemcpyAsync(npat_dev, gid + n - 1, 4, cudaMemcpyDeviceToDevice, s));
    // rep reuses the key buffer (n words); frequencies start at zero.
    uint32_t *rep = reinterpret_cast<uint32_t *>(k0);
    CXG_CUDA(cudaMemsetAsync(freq_out, 0, n * 4, s));
    compact_scatter<<<nb, 256, 0, s>>>(i0, flag, gid, (unsigned)n, freq_in, rep, freq_out);
    CXG_CHECK_LAUNCH("compact_scatter");
    const unsigned wide = mstride > nsites ? mstride : nsites;
    dim3 eg((wide + 255) / 256, ntaxa);
    compact_emit<<<eg, 256, 0, s>>>(rows, ntaxa, nsites, rep, npat_dev, canon, val, any_mask,
                                    rows_out, rstride, masks, mstride);
    CXG_CHECK_LAUNCH("compact_emit");
    return 0;
}

}  // namespace cxg

using namespace cxg;

static std::mutex g_compact_mu;

extern "C" int cxgCompact(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                          const uint32_t *freqs, const uint8_t *canon, const uint8_t *val,
                          uint8_t any_mask, uint8_t *rows_out, uint32_t *freqs_out,
                          uint8_t *masks_out, unsigned *npat) {
    if (rows == nullptr || canon == nullptr || npat == nullptr || freqs_out == nullptr)
        return fail(CXG_EINVAL, "cxgCompact: NULL");
    if (masks_out && val == nullptr) return fail(CXG_EINVAL, "cxgCompact: masks need val");
    if (ntaxa == 0) return fail(CXG_EINVAL, "cxgCompact: no taxa");
    if (nsites == 0) {
        *npat = 0;
        return 0;
    }
    std::lock_guard<std::mutex> lk(g_compact_mu);
    const size_t in_bytes = (size_t)ntaxa * nsites;
    const size_t work = compact_work_bytes(ntaxa, nsites);
    const size_t o_rows = 0, o_freq = al256c(in_bytes), o_tab = o_freq + al256c((size_t)nsites * 4);
    const size_t o_out = o_tab + 1024, o_fout = o_out + al256c(in_bytes);
    const size_t o_mask = o_fout + al256c((size_t)nsites * 4), o_np = o_mask + al256c(in_bytes);
    const size_t o_work = o_np + 256;
    char *d = nullptr;
    cudaStream_t s = nullptr;
    CXG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaError_t e = cudaMallocAsync((void **)&d, o_work + work, s);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return cuda_fail(e, "cxgCompact: device memory");
    }
    int rc = 0;
    auto fin = [&](int r) {
        cudaFreeAsync(d, s);
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
        return r;
    };
    uint8_t tabs[768];
    memset(tabs, 0, 256);
    memcpy(tabs + 256, canon, 256);
    if (val) memcpy(tabs + 512, val, 256); else memset(tabs + 512, 0, 256);
    if ((e = cudaMemcpyAsync(d + o_rows, rows, in_bytes, cudaMemcpyHostToDevice, s)) ||
        (freqs && (e = cudaMemcpyAsync(d + o_freq, freqs, (size_t)nsites * 4,
                                       cudaMemcpyHostToDevice, s))) ||
        (e = cudaMemcpyAsync(d + o_tab, tabs, 768, cudaMemcpyHostToDevice, s)))
        return fin(cuda_fail(e, "cxgCompact: upload"));
    const uint8_t *dt = (const uint8_t *)(d + o_tab);
    rc = compact_device((const uint8_t *)(d + o_rows), ntaxa, nsites,
                        freqs ? (const uint32_t *)(d + o_freq) : nullptr, canon, dt + 256,
                        dt + 512, any_mask, (uint8_t *)(d + o_out), nsites,
                        masks_out ? (uint8_t *)(d + o_mask) : nullptr, nsites,
                        (uint32_t *)(d + o_fout), (uint32_t *)(d + o_np), d + o_work, work, s);
    if (rc) return fin(rc);
    uint32_t np = 0;
    if ((e = cudaMemcpyAsync(&np, d + o_np, 4, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return fin(cuda_fail(e, "cxgCompact: pattern count"));
    // Rows and masks come back with row stride npat.
    if (rows_out && np &&
        (e = cudaMemcpy2DAsync(rows_out, np, d + o_out, nsites, np, ntaxa,
                               cudaMemcpyDeviceToHost, s)))
        return fin(cuda_fail(e, "cxgCompact: rows"));
    if (masks_out && np &&
        (e = cudaMemcpy2DAsync(masks_out, np, d + o_mask, nsites, np, ntaxa,
                               cudaMemcpyDeviceToHost, s)))
        return fin(cuda_fail(e, "cxgCompact: masks"));
    if ((e = cudaMemcpyAsync(freqs_out, d + o_fout, (size_t)np * 4, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return fin(cuda_fail(e, "cxgCompact: frequencies"));
    *npat = np;
    return fin(0);
}
