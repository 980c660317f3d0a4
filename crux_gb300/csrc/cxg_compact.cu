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
//      index) pairs (cub::DeviceRadixSort, a CUDA toolkit primitive).
//   3. compact_flags: a column starts a pattern unless all its chunk keys
//      equal those of the column before it (the packing is exact); a scan
//      numbers the patterns.
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
    size_t cub_bytes = 0, scan_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, (const unsigned long long *)nullptr,
                                    (unsigned long long *)nullptr, (const uint32_t *)nullptr,
                                    (uint32_t *)nullptr, (int)nsites);
    cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, (const uint32_t *)nullptr,
                                  (uint32_t *)nullptr, (int)nsites);
    const size_t n = nsites;
    return 2048 + al256c(max_chunks * n * 8) + 2 * al256c(n * 8) + 4 * al256c(n * 4) +
           al256c(cub_bytes > scan_bytes ? cub_bytes : scan_bytes);
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
    size_t cub_bytes = work_bytes - (size_t)(p - static_cast<char *>(work));
    void *cub_tmp = p;

    const unsigned nb = (unsigned)((n + 255) / 256);
    compact_keys<<<dim3(nb, nchunks), 256, 0, s>>>(rows, ntaxa, nsites, rank, bits, cpk, keys);
    CXG_CHECK_LAUNCH("compact_keys");
    // Identity order, then one stable sort per key chunk, last chunk first.
    std::vector<uint32_t> iota(n);
    for (size_t i = 0; i < n; ++i) iota[i] = (uint32_t)i;
    CXG_CUDA(cudaMemcpyAsync(i0, iota.data(), n * 4, cudaMemcpyHostToDevice, s));
    for (int c = (int)nchunks - 1; c >= 0; --c) {
        compact_gather<<<nb, 256, 0, s>>>(keys + (size_t)c * n, i0, (unsigned)n, k0);
        CXG_CHECK_LAUNCH("compact_gather");
        cudaError_t e = cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, k0, k1, i0, i1,
                                                        (int)n, 0, (int)(cpk * bits), s);
        if (e != cudaSuccess) return cuda_fail(e, "compaction radix sort");
        uint32_t *t = i0;
        i0 = i1;
        i1 = t;
    }
    compact_flags<<<nb, 256, 0, s>>>(keys, nchunks, i0, (unsigned)n, flag);
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
        cudaFreeHost(p);
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
        cudaFreeAsync(d, s);
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
