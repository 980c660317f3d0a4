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
//   1. compact_keys: every column's characters, `cpk` to a 64-bit key
//      (first character most significant, rank order = byte order), as
//      key[chunk][site], read straight from the row-major input.
//   2. LSD sort: for each chunk, last first, gather the chunk key of every
//      column in the current order and stable-radix-sort (key, column
//      index) pairs: 8-bit digits, each a histogram per tile, one scan of
//      the (digit, tile) counts and a stable scatter (radix_hist,
//      radix_scan, radix_scatter below).
//   3. compact_flags: a column starts a pattern unless all its chunk keys
//      equal those of the column before it (the packing is exact); a scan
//      numbers the patterns.
//   4. compact_scatter / compact_emit: the first column of each pattern
//      represents it, frequencies add (integer atomics: exact), and the
//      canonical rows and state masks of the patterns are written.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "cxg_internal.h"

namespace cxg {
namespace {

// used[c] = 1 for every canonical code c that occurs.  Rows are read 16
// bytes a thread (the input is a device allocation, 16-byte aligned).
__global__ void compact_used(const uint8_t *rows, size_t n, const uint8_t *canon,
                             uint32_t *used) {
    __shared__ uint32_t u[256];
    __shared__ uint8_t cs[256];
    for (unsigned i = threadIdx.x; i < 256; i += blockDim.x) {
        u[i] = 0;
        cs[i] = canon[i];
    }
    __syncthreads();
    const size_t n16 = n / 16;
    const uint4 *r16 = reinterpret_cast<const uint4 *>(rows);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16;
         i += (size_t)gridDim.x * blockDim.x) {
        const uint4 v = __ldg(r16 + i);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int b = 0; b < 4; ++b) u[cs[(w[q] >> (8 * b)) & 255u]] = 1;
    }
    for (size_t i = n16 * 16 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        u[cs[rows[i]]] = 1;
    __syncthreads();
    for (unsigned i = threadIdx.x; i < 256; i += blockDim.x)
        if (u[i]) used[i] = 1;
}

// keys[c][s] = ranks of characters [c*cpk, c*cpk + cpk) of column s,
// `bits` bits each, the first one most significant (rank 0 past ntaxa).
// Thread per site: each character read is a coalesced row access.
__global__ void compact_keys(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                             const uint8_t *rank, unsigned bits, unsigned cpk,
                             unsigned long long *keys) {
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned c = blockIdx.y;
    if (s >= nsites) return;
    unsigned long long k = 0;
    for (unsigned j = 0; j < cpk; ++j) {
        const unsigned t = c * cpk + j;
        k = (k << bits) | (t < ntaxa ? rank[rows[(size_t)t * nsites + s]] : 0u);
    }
    keys[(size_t)c * nsites + s] = k;
}

// key[i] = keys[c][idx[i]]: chunk c of the columns in the current order.
__global__ void compact_gather(const unsigned long long *keys_c, const uint32_t *idx,
                               unsigned n, unsigned long long *key) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) key[i] = keys_c[idx[i]];
}

// flag[i] = 1 if column idx[i] differs from column idx[i - 1] (or i == 0):
// some chunk key differs.
__global__ void compact_flags(const unsigned long long *keys, unsigned nchunks,
                              const uint32_t *idx, unsigned n, uint32_t *flag) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i == 0) {
        flag[0] = 1;
        return;
    }
    const size_t a = idx[i], b = idx[i - 1];
    uint32_t diff = 0;
    for (unsigned c = 0; c < nchunks && !diff; ++c)
        diff = keys[(size_t)c * n + a] != keys[(size_t)c * n + b];
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

// --- stable LSD radix sort of (64-bit key, 32-bit value) pairs ------------
// One pass orders the pairs by the 8-bit digit (key >> shift) & 255, keeping
// the order of equal digits.  The input is cut into tiles of kSortTile
// pairs, one CTA each.
constexpr unsigned kSortThreads = 256;
constexpr unsigned kSortTile = 1024;

// hist[d * ntiles + b] = pairs of tile b with digit d.
__global__ void __launch_bounds__(kSortThreads)
    radix_hist(const unsigned long long *key, unsigned n, unsigned shift, uint32_t *hist) {
    __shared__ uint32_t h[256];
    const unsigned t = threadIdx.x;
    h[t] = 0;
    __syncthreads();
    const unsigned base = blockIdx.x * kSortTile;
    const unsigned end = min(base + kSortTile, n);
    for (unsigned i = base + t; i < end; i += kSortThreads)
        atomicAdd(&h[(unsigned)(key[i] >> shift) & 255u], 1u);
    __syncthreads();
    hist[t * gridDim.x + blockIdx.x] = h[t];
}

// Exclusive scan of the NT values v[0..n) in place, one CTA of NT
// threads: each thread sums a contiguous segment, the segment sums are
// scanned in shared memory, then each thread writes its segment's
// prefixes.  Returns the total (every thread).
template <unsigned NT>
__device__ uint32_t block_exclusive_scan(uint32_t *v, unsigned n) {
    __shared__ uint32_t part[NT];
    const unsigned t = threadIdx.x;
    const unsigned seg = (n + NT - 1) / NT;
    const unsigned a = min(t * seg, n), b = min(a + seg, n);
    uint32_t sum = 0;
    for (unsigned i = a; i < b; ++i) sum += v[i];
    part[t] = sum;
    __syncthreads();
    for (unsigned off = 1; off < NT; off <<= 1) {
        const uint32_t x = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;  // exclusive prefix of this segment
    for (unsigned i = a; i < b; ++i) {
        const uint32_t x = v[i];
        v[i] = run;
        run += x;
    }
    const uint32_t total = part[NT - 1];
    __syncthreads();  // part is reused by the next call
    return total;
}

// Exclusive scan of v[0..n) in place, one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) radix_scan(uint32_t *v, unsigned n) {
    block_exclusive_scan<1024>(v, n);
}

// Digit d's row of tile counts, hist[d * ntiles ..], scanned in place by
// CTA d; tot[d] = the digit's count.
__global__ void __launch_bounds__(kSortThreads)
    radix_rowscan(uint32_t *hist, unsigned ntiles, uint32_t *tot) {
    const uint32_t t = block_exclusive_scan<kSortThreads>(hist + (size_t)blockIdx.x * ntiles,
                                                          ntiles);
    if (threadIdx.x == 0) tot[blockIdx.x] = t;
}

// Stable scatter of one pass.  A tile is read in rounds of kSortThreads
// pairs, pair r + t to thread t, so lower threads hold earlier pairs.  A
// pair's place is its digit's next free slot for this tile (offs: the
// digit's base, an exclusive scan of the digit counts tot, plus its
// row-scanned tile count), plus the pairs with its digit in lower warps of
// the round (wcnt) and in lower lanes of its warp (__match_any_sync).
__global__ void __launch_bounds__(kSortThreads)
    radix_scatter(const unsigned long long *kin, const uint32_t *vin, unsigned n,
                  unsigned shift, const uint32_t *hist, const uint32_t *tot,
                  unsigned long long *kout, uint32_t *vout) {
    constexpr unsigned W = kSortThreads / 32;
    __shared__ uint32_t offs[256];
    __shared__ uint32_t wcnt[W][256];
    const unsigned t = threadIdx.x, w = t / 32, lane = t % 32;
    offs[t] = tot[t];
    __syncthreads();
    block_exclusive_scan<kSortThreads>(offs, 256);
    offs[t] += hist[t * gridDim.x + blockIdx.x];
    for (unsigned j = 0; j < W; ++j) wcnt[j][t] = 0;
    __syncthreads();
    const unsigned base = blockIdx.x * kSortTile;
    const unsigned end = min(base + kSortTile, n);
    for (unsigned r = base; r < end; r += kSortThreads) {
        const unsigned i = r + t;
        const bool active = i < end;
        const unsigned long long k = active ? kin[i] : 0ull;
        const uint32_t v = active ? vin[i] : 0u;
        // Inactive lanes get a digit no other lane has.
        const unsigned d = active ? ((unsigned)(k >> shift) & 255u) : 256u + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned below = __popc(peers & ((1u << lane) - 1u));
        const bool leader = below == 0;
        if (active && leader) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (active) {
            unsigned pos = offs[d] + below;
            for (unsigned j = 0; j < w; ++j) pos += wcnt[j][d];
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
        if (active && leader) {
            atomicAdd(&offs[d], __popc(peers));
            wcnt[w][d] = 0;
        }
        __syncthreads();
    }
}

// Inclusive scan of n values (in and out may not alias), by tiles of 1024:
// tile sums, an exclusive scan of those (radix_scan), then each tile's
// inclusive scan plus its offset.
__global__ void __launch_bounds__(1024)
    tile_sums(const uint32_t *in, unsigned n, uint32_t *sums) {
    __shared__ uint32_t ws[32];
    const unsigned i = blockIdx.x * 1024 + threadIdx.x;
    uint32_t x = i < n ? in[i] : 0u;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x / 32] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        x = ws[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = x;
    }
}

__global__ void __launch_bounds__(1024)
    tile_scan(const uint32_t *in, unsigned n, const uint32_t *offs, uint32_t *out) {
    __shared__ uint32_t ws[32];
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x / 32;
    const unsigned i = blockIdx.x * 1024 + threadIdx.x;
    uint32_t x = i < n ? in[i] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t y = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= (unsigned)o) y += z;
        }
        ws[lane] = y;
    }
    __syncthreads();
    if (i < n) out[i] = x + (w ? ws[w - 1] : 0u) + offs[blockIdx.x];
}

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
    // Chunk keys for the widest ranks (8 bits: 8 characters a key).
    const size_t max_chunks = (ntaxa + 7) / 8;
    const size_t n = nsites;
    const size_t ntiles = (n + kSortTile - 1) / kSortTile;
    const size_t hist = ntiles * 256 * 4 + 1024, scan = ((n + 1023) / 1024) * 4;
    return 2048 + al256c(max_chunks * n * 8) + 2 * al256c(n * 8) + 4 * al256c(n * 4) +
           al256c(hist > scan ? hist : scan);
}

int compact_device(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                   const uint32_t *freq_in, const uint8_t *canon_host, const uint8_t *canon,
                   const uint8_t *val, uint8_t any_mask, uint8_t *rows_out, unsigned rstride,
                   uint8_t *masks, unsigned mstride, uint32_t *freq_out, uint32_t *npat_dev,
                   void *work, size_t work_bytes, cudaStream_t s) {
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
    const unsigned cpk = 64 / bits;
    const unsigned nchunks = (ntaxa + cpk - 1) / cpk;
    if (nchunks > 65535) return fail(CXG_EINVAL, "compaction: too many taxa");
    unsigned long long *keys = (unsigned long long *)take(((size_t)ntaxa + 7) / 8 * n * 8);
    unsigned long long *k0 = (unsigned long long *)take(n * 8);
    unsigned long long *k1 = (unsigned long long *)take(n * 8);
    uint32_t *i0 = (uint32_t *)take(n * 4);
    uint32_t *i1 = (uint32_t *)take(n * 4);
    uint32_t *flag = (uint32_t *)take(n * 4);
    uint32_t *gid = (uint32_t *)take(n * 4);
    const unsigned ntiles = (unsigned)((n + kSortTile - 1) / kSortTile);
    uint32_t *hist = (uint32_t *)p;  // [256][ntiles] digit counts, or tile sums
    uint32_t *dtot = hist + (size_t)ntiles * 256;  // [256] counts of each digit

    const unsigned nb = (unsigned)((n + 255) / 256);
    compact_keys<<<dim3(nb, nchunks), 256, 0, s>>>(rows, ntaxa, nsites, rank, bits, cpk, keys);
    CXG_CHECK_LAUNCH("compact_keys");
    // Identity order, then one stable sort per key chunk, last chunk first.
    std::vector<uint32_t> iota(n);
    for (size_t i = 0; i < n; ++i) iota[i] = (uint32_t)i;
    CXG_CUDA(cudaMemcpyAsync(i0, iota.data(), n * 4, cudaMemcpyHostToDevice, s));
    const unsigned kbits = cpk * bits;
    for (int c = (int)nchunks - 1; c >= 0; --c) {
        compact_gather<<<nb, 256, 0, s>>>(keys + (size_t)c * n, i0, (unsigned)n, k0);
        CXG_CHECK_LAUNCH("compact_gather");
        // Stable passes over the key's 8-bit digits, least significant first.
        for (unsigned shift = 0; shift < kbits; shift += 8) {
            radix_hist<<<ntiles, kSortThreads, 0, s>>>(k0, (unsigned)n, shift, hist);
            radix_rowscan<<<256, kSortThreads, 0, s>>>(hist, ntiles, dtot);
            radix_scatter<<<ntiles, kSortThreads, 0, s>>>(k0, i0, (unsigned)n, shift, hist,
                                                          dtot, k1, i1);
            CXG_CHECK_LAUNCH("compaction radix sort");
            unsigned long long *tk = k0;
            k0 = k1;
            k1 = tk;
            uint32_t *ti = i0;
            i0 = i1;
            i1 = ti;
        }
    }
    compact_flags<<<nb, 256, 0, s>>>(keys, nchunks, i0, (unsigned)n, flag);
    CXG_CHECK_LAUNCH("compact_flags");
    // gid = inclusive scan of the flags.
    const unsigned nt = (unsigned)((n + 1023) / 1024);
    tile_sums<<<nt, 1024, 0, s>>>(flag, (unsigned)n, hist);
    radix_scan<<<1, 1024, 0, s>>>(hist, nt);
    tile_scan<<<nt, 1024, 0, s>>>(flag, (unsigned)n, hist, gid);
    CXG_CHECK_LAUNCH("compaction scan");
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

// Copies between pageable host arrays and the device go through two pinned
// chunks (allocated once, kept, guarded by g_compact_mu): the host copies
// one chunk while the DMA engine moves the other.  Pageable copies run at a
// small fraction of the DMA rate.
namespace {
constexpr size_t kStageChunk = (size_t)32 << 20;
unsigned char *g_stage[2] = {nullptr, nullptr};
cudaEvent_t g_stage_ev[2] = {nullptr, nullptr};

int stage_init() {
    if (g_stage[0]) return 0;
    unsigned char *p = nullptr;
    CXG_CUDA(host_alloc((void **)&p, 2 * kStageChunk));
    cudaError_t e = cudaEventCreateWithFlags(&g_stage_ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g_stage_ev[1], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        host_free(p);
        return cuda_fail(e, "cxgCompact: staging events");
    }
    g_stage[0] = p;
    g_stage[1] = p + kStageChunk;
    return 0;
}

int staged_h2d(void *dst, const void *src, size_t n, cudaStream_t s) {
    const unsigned char *h = static_cast<const unsigned char *>(src);
    unsigned char *d = static_cast<unsigned char *>(dst);
    for (size_t off = 0, i = 0; off < n; off += kStageChunk, ++i) {
        const int b = (int)(i & 1);
        const size_t len = n - off < kStageChunk ? n - off : kStageChunk;
        CXG_CUDA(cudaEventSynchronize(g_stage_ev[b]));  // its last DMA is done
        memcpy(g_stage[b], h + off, len);
        CXG_CUDA(cudaMemcpyAsync(d + off, g_stage[b], len, cudaMemcpyHostToDevice, s));
        CXG_CUDA(cudaEventRecord(g_stage_ev[b], s));
    }
    return 0;
}

// height rows of `width` bytes, device pitch dpitch, into host rows of
// pitch `width`.
int staged_d2h_rows(void *dst, const void *src, size_t dpitch, size_t width, size_t height,
                    cudaStream_t s) {
    unsigned char *h = static_cast<unsigned char *>(dst);
    const unsigned char *d = static_cast<const unsigned char *>(src);
    if (width > kStageChunk) {
        CXG_CUDA(cudaMemcpy2DAsync(h, width, d, dpitch, width, height, cudaMemcpyDeviceToHost,
                                   s));
        CXG_CUDA(cudaStreamSynchronize(s));
        return 0;
    }
    const size_t per = kStageChunk / width;
    const size_t nblk = (height + per - 1) / per;
    auto issue = [&](size_t k) -> int {
        const size_t r0 = k * per, nr = height - r0 < per ? height - r0 : per;
        const int b = (int)(k & 1);
        CXG_CUDA(cudaMemcpy2DAsync(g_stage[b], width, d + r0 * dpitch, dpitch, width, nr,
                                   cudaMemcpyDeviceToHost, s));
        CXG_CUDA(cudaEventRecord(g_stage_ev[b], s));
        return 0;
    };
    if (int rc = issue(0)) return rc;
    for (size_t k = 0; k < nblk; ++k) {
        if (k + 1 < nblk)
            if (int rc = issue(k + 1)) return rc;
        const int b = (int)(k & 1);
        CXG_CUDA(cudaEventSynchronize(g_stage_ev[b]));
        const size_t r0 = k * per, nr = height - r0 < per ? height - r0 : per;
        memcpy(h + r0 * width, g_stage[b], nr * width);
    }
    return 0;
}
}  // namespace

extern "C" int cxgCompact(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                          const uint32_t *freqs, const uint8_t *canon, const uint8_t *val,
                          uint8_t any_mask, uint8_t *rows_out, uint32_t *freqs_out,
                          uint8_t *masks_out, unsigned *npat) {
    NvtxRange nr("cxgCompact");
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
    cudaError_t e = dev_malloc_async((void **)&d, o_work + work, s);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return cuda_fail(e, "cxgCompact: device memory");
    }
    int rc = 0;
    auto fin = [&](int r) {
        dev_free_async(d, s);
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
        return r;
    };
    uint8_t tabs[768];
    memset(tabs, 0, 256);
    memcpy(tabs + 256, canon, 256);
    if (val) memcpy(tabs + 512, val, 256); else memset(tabs + 512, 0, 256);
    if ((rc = stage_init()) || (rc = staged_h2d(d + o_rows, rows, in_bytes, s))) return fin(rc);
    if ((freqs && (e = cudaMemcpyAsync(d + o_freq, freqs, (size_t)nsites * 4,
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
    if (rows_out && np && (rc = staged_d2h_rows(rows_out, d + o_out, nsites, np, ntaxa, s)))
        return fin(rc);
    if (masks_out && np && (rc = staged_d2h_rows(masks_out, d + o_mask, nsites, np, ntaxa, s)))
        return fin(rc);
    if ((e = cudaMemcpyAsync(freqs_out, d + o_fout, (size_t)np * 4, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return fin(cuda_fail(e, "cxgCompact: frequencies"));
    *npat = np;
    return fin(0);
}
