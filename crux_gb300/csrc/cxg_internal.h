// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "cxlik_gpu.h"
#include <nvtx3/nvToolsExt.h>

namespace cxg {

// An NVTX range over one library call (header-only NVTX: a no-op unless a
// profiler is attached), so that a trace or an `ncu --nvtx` filter can
// tell the calls apart.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Patterns are padded to a multiple of this on the device, so that every
// plane of a CL buffer starts on a 512-byte boundary.
constexpr unsigned kPatternQuantum = 128;
// Most patterns per tile.
constexpr unsigned kBlock = 128;
// Largest CTA of the plan walkers: tile patterns x threads per pattern.
constexpr unsigned kMaxThreads = 256;
// Largest CTA of the op-lane walker: 2 lanes x tile patterns (tile <= 64).
constexpr unsigned kLaneThreads = 128;
// Default patterns per tile.
constexpr unsigned kTile = 64;
// Most shared-memory stack slots per tile.
constexpr unsigned kMaxSlots = 16;
// Op records in flight per CTA (bulk-copy ring depth).
constexpr unsigned kRing = 4;
// Default iteration bound of every spin on an mbarrier (the record waits
// take theirs from set_spin_limit).
constexpr unsigned kSpinLimit = 1u << 26;
// Largest number of active mixture components held in registers.
constexpr unsigned kMaxComps = 8;
// Largest node degree handled in one op (children per parent).
constexpr unsigned kMaxChildren = 16;

inline unsigned pad_patterns(unsigned p) {
    return (p + kPatternQuantum - 1) / kPatternQuantum * kPatternQuantum;
}

// Where a child's CL comes from during a plan walk.
enum : uint32_t {
    SRC_GLOBAL = 0,  // internal CL in HBM, computed by an earlier run
    SRC_LEAF = 1,    // leaf masks, staged in shared memory per tile
    SRC_SLOT = 2     // internal CL produced earlier in this run, still held
                     // in the tile's shared-memory stack slot `idx`
};

// Op records.  The host packs every node update of a plan into one
// fixed-stride record (rstride bytes, a multiple of 16), so that a CTA can
// stream the records into shared memory with bulk copies ahead of use:
//
//   RecHead | RecChild[nchild] | one area per child, at RecChild.off
//
// A child's area is filled in place by the P-matrix kernel of each run:
// the P matrices T P[kact][16], or for a leaf child of an FP32 plan its
// message table float[kact][16 masks][4] (the message P x indicator(mask)
// of every state mask, summed in FP64 and rounded once).
struct RecHead {
    void *data;        // parent CL in HBM, [K][U][ppad] 16-byte units
    void *scaler;      // parent scaler [ppad]
    uint32_t nchild;
    int32_t slot;      // stack slot keeping the result for a later op, or -1
    uint32_t flags;    // REC_NO_HBM: the result is not written to HBM
    // Bytes of the record `ring` positions later, which refills this ring
    // stage after this op (a multiple of 16); 0: the whole record stride.
    // Read by the one-lane walker with staged leaves; others copy whole
    // strides.
    uint32_t next_bytes;
};

// RecHead.flags: the parent is consumed from its stack slot (or is the
// root) and is not kept as a cache, so the walker skips its HBM write.
enum : uint32_t { REC_NO_HBM = 1 };

// RecHead.flags bits 8-10: the kind of a two-child op of an FP32 plan run
// one op at a time, one thread per pattern, named by where its children
// come from (F: the previous op's result, still in registers; L: a leaf;
// I: an internal CL in HBM or a stack slot).  The walker then runs
// straight-line code for that kind.  Bit 12 gives the record index of
// child A (the first letter); child B is the other.  A product of two
// messages and a sum of two integer exponents are the same in either
// order, so the kind's A/B order gives the bits of the record order.
// OPK_GENERIC (0) runs the general per-child loop.
enum : uint32_t {
    OPK_GENERIC = 0,
    OPK_FL = 1,
    OPK_FI = 2,
    OPK_LL = 3,
    OPK_IL = 4,
    OPK_II = 5
};
constexpr uint32_t kOpKindShift = 8;
constexpr uint32_t kOpKindA = 1u << 12;

// RecHead.flags bits of a two-child op whose children are of classes a and
// b (0: L, 1: I, 2: F).  A is the child of the higher class.
__host__ __device__ inline uint32_t op_kind_of_classes(int a, int b) {
    if (a == 2 && b == 2) return 0;  // not a plan
    const int hi = a > b ? a : b, lo = a > b ? b : a;
    const uint32_t ia = (a >= b) ? 0u : kOpKindA;
    uint32_t kind = OPK_GENERIC;
    if (hi == 2) kind = lo == 0 ? OPK_FL : OPK_FI;
    else if (hi == 1) kind = lo == 0 ? OPK_IL : OPK_II;
    else kind = OPK_LL;
    return (kind << kOpKindShift) | ia;
}

// The same for children with sources src0 / src1 and HBM rows data0 /
// data1, in an op run right after the op whose result is `prev` (null for
// the first op): a child is F when it is that result, which the walker
// still holds in registers.
__host__ __device__ inline uint32_t op_kind_flags(uint32_t src0, const void *data0,
                                                  uint32_t src1, const void *data1,
                                                  const void *prev) {
    auto cls = [&](uint32_t src, const void *d) {
        return src == SRC_LEAF ? 0 : (prev != nullptr && d == prev ? 2 : 1);
    };
    return op_kind_of_classes(cls(src0, data0), cls(src1, data1));
}

// One child of an op.  `data`/`scaler` address the HBM copy (SRC_GLOBAL);
// for SRC_LEAF `data` is the leaf's mask array [ppad] (one uint8 state
// mask per pattern) and `idx` its staged row when the job stages leaves;
// for SRC_SLOT `idx` is the stack slot.
struct RecChild {
    const void *data;
    const void *scaler;
    uint32_t src;
    uint32_t idx;
    uint32_t tab;      // FP64 plans: leaf-message table of this child
    uint32_t off;      // byte offset of the child's area in the record
};

// Bytes of a child's area in an op record.
__host__ __device__ inline size_t child_area_bytes(int precision, unsigned kact,
                                                   bool leaf) {
    if (precision == CXG_FP32 && leaf) return (size_t)16 * kact * 4 * 4;
    return (size_t)kact * 16 * (precision == CXG_FP32 ? 4 : 8);
}

static_assert(sizeof(RecHead) == 32, "record header is 32 bytes");
static_assert(sizeof(RecChild) == 32, "record child is 32 bytes");

// Per-call constants of a plan execution.  CL buffers in HBM are
// [K][U][ppad] 16-byte units (U = 1 for FP32: states 0-3; U = 2 for FP64:
// states 0-1, 2-3), so that one thread per pattern moves whole units and a
// warp writes 512 contiguous bytes per store.
struct PlanArgs {
    const unsigned char *rec;      // [nops][rstride] op records
    // [nops][lmax] mask arrays of each op's leaf children, in the record's
    // child order, null-terminated when fewer than lmax: they are copied
    // with the op's record, so lmax rows of tile bytes follow it in the
    // stage (a plan with no leaf children may use lmax 0).
    const uint8_t *const *lrows;
    uint32_t lmax;
    // A job whose leaves fit the staging budget stages them instead: nleaf
    // mask arrays, each loaded once per tile; leaf children then name their
    // staged row by RecChild.idx (lmax is 0).  nleaf 0: leaves stream.
    const uint8_t *const *leaves;
    uint32_t nleaf;
    uint32_t rstride;
    uint32_t ring;        // records in flight per CTA
    uint32_t nops;
    uint32_t nslot;       // shared-memory stack slots per tile
    uint32_t tile;        // patterns per CTA (blockDim.x / tpp)
    uint32_t kact;        // active components (weightScaled != 0)
    uint32_t npat;        // patterns (mschars)
    uint32_t ppad;        // padded pattern stride
    uint32_t root_last;   // the last op writes the root CL
    const double *pn;     // [kact][4] pi_i * weightScaled (root weights)
    const void *root;     // root CL buffer
    const void *rootsc;   // root scaler
    const uint32_t *freqs;// [npat] pattern weights (charFreqs + cbase)
    double *site;         // [npat] site lnL out (may be null)
    double *partial;      // [nblocks][2] compensated partial sums
    uint32_t *ninf;       // count of -inf sites
    unsigned *ticket;     // last-block counter
    double *total;        // [2] final (sum, compensation)
    uint32_t *err;        // nonzero: a bounded wait gave up
    const double *ltab;   // FP64 plans: [ntab][16 masks][kact][4]
    uint32_t ntiles;      // tiles of this job (ppad / tile)
    uint32_t no_root;     // 1: stop after the ops (per-node launches)
    uint32_t tpp;         // threads per pattern (each holds kact / tpp
                          // components); 0 is read as 1
    uint32_t ppt;         // patterns per thread (1 or 2); 0 is read as 1
};

// Threads per pattern and patterns per thread a walker is built for with
// `kact` components: one of each for every shape; 2 or 4 threads per
// pattern for the FP32 form when they divide kact; 2 patterns per thread
// for the FP32 form with one thread per pattern and at most 5 components.
// Op lanes (two independent ops per step, walk_tile's L) exist for the
// FP32 form with one thread and one pattern per thread, kact <= 5.
inline bool lanes_shape_ok(int precision, unsigned kact, unsigned tpp, unsigned ppt) {
    return precision == CXG_FP32 && tpp == 1 && ppt == 1 && kact >= 1 && kact <= 5;
}

inline bool walker_shape_ok(int precision, unsigned kact, unsigned tpp,
                            unsigned ppt = 1) {
    if (ppt == 2)
        return precision == CXG_FP32 && tpp == 1 && kact >= 1 && kact <= 5;
    if (ppt != 1) return false;
    if (tpp == 1) return kact >= 1 && kact <= kMaxComps;
    if (precision != CXG_FP32 || (tpp != 2 && tpp != 4)) return false;
    return kact % tpp == 0 && kact / tpp <= (tpp == 2 ? 4u : 2u);
}

// Threads per pattern for a new plan: the tuned value where the walker is
// built for it (walker_shape_ok, tile x tpp <= kMaxThreads), else 1.
inline unsigned tuned_tpp(int precision, unsigned kact, unsigned tile) {
    unsigned t = 0, tpp = 1, ppt = 1;
    size_t b = 0;
    cxgTuneGet(&t, &tpp, &ppt, &b);
    if (!walker_shape_ok(precision, kact, tpp) || tile * tpp > kMaxThreads) tpp = 1;
    return tpp;
}

// Patterns per thread for a new plan with `tpp` threads per pattern: the
// tuned value where the walker is built for it (and the tile keeps at
// least one warp), else 1.
inline unsigned tuned_ppt(int precision, unsigned kact, unsigned tile, unsigned tpp) {
    unsigned t = 0, tq = 1, ppt = 1;
    size_t b = 0;
    cxgTuneGet(&t, &tq, &ppt, &b);
    if (!walker_shape_ok(precision, kact, tpp, ppt) || tile / ppt < 32) ppt = 1;
    return ppt;
}

// One (job, tile) work item of a batched launch.
struct WalkItem {
    uint32_t job;
    uint32_t tile;
};

// A batched launch: a persistent grid claims items from `counter` (items
// sorted longest first by the host); shared memory is laid out for the
// largest job (nslot, rstride and lmax maxima); all jobs share kact, tile and
// the ring depth.
struct BatchArgs {
    const PlanArgs *jobs;
    const WalkItem *items;
    uint32_t nitems;
    unsigned *counter;
    uint32_t tile, ring, kact;
    uint32_t max_nslot, max_rstride, max_lmax, max_nleaf;
    uint32_t tpp;         // threads per pattern (all jobs); 0 is read as 1
    uint32_t ppt;         // patterns per thread (all jobs); 0 is read as 1
    uint32_t direct;      // 1: CTA i walks item i (grid = nitems), no
                          // counter; launch_batch sets it
};

size_t plan_smem_bytes(int precision, unsigned kact, unsigned tile, unsigned nslot,
                       unsigned ring, unsigned rstride, unsigned lmax,
                       unsigned nleaf);
// Pattern compression on the device (cxg_compact.cu): scratch bytes, and
// the compaction of rows [ntaxa][nsites] (device, 16-byte aligned) into rows_out / masks
// (row strides rstride / mstride; mask pad patterns up to mstride get
// any_mask), freq_out and *npat_dev (device).  canon_host is the host copy
// of the device table canon.  Waits for the stream once.
size_t compact_work_bytes(unsigned ntaxa, unsigned nsites);
int compact_device(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
                   const uint32_t *freq_in, const uint8_t *canon_host, const uint8_t *canon,
                   const uint8_t *val, uint8_t any_mask, uint8_t *rows_out, unsigned rstride,
                   uint8_t *masks, unsigned mstride, uint32_t *freq_out, uint32_t *npat_dev,
                   void *work, size_t work_bytes, cudaStream_t s);

// Largest staged leaf rows per CTA: jobs whose leaves take more stream
// them with their records instead.
constexpr size_t kLeafStageBytes = 16 * 1024;
cudaError_t launch_batch(int precision, const BatchArgs &b, unsigned grid,
                         cudaStream_t s);
// Resident CTAs per SM of the batched walker for this shape.
int batch_ctas_per_sm(int precision, unsigned kact, unsigned tile,
                      unsigned tpp, unsigned ppt, bool staged, size_t smem);

// Inputs of the P-matrix kernel: one thread per (child, active comp); the
// P matrix (FP64 arithmetic, stored as the plan's precision) goes into the
// child's op record at byte offset dst[child] + k * 16 * sizeof(T).
struct PmatArgs {
    uint32_t nchild;
    uint32_t kact;
    int precision;
    const double *edge_len;    // [nchild]
    const double *cmult;       // [kact]
    const double *rmult;       // [kact]
    const int32_t *model;      // [kact] model index of each active comp
    const double *cube;        // [nmodels][64]
    const double *eig;         // [nmodels][4]
    const uint64_t *dst;       // [nchild] byte offsets from rec
    const int32_t *tab;        // [nchild] leaf child: FP64 table index (FP32:
                               // any value >= 0, the table goes in the record); -1
    double wnorm;
    const double *wnorm_dev;   // if set, wNorm is read here (model built on the GPU)
    unsigned char *rec;
    double *ltab;              // FP64 plans: leaf-message tables
    uint64_t *zero = nullptr;  // pmat_kernel: four words cleared before the
                               // walker that follows it runs (its result)
};

// Allocations of the library (cxg_lik.cu); each fails as an out-of-memory
// would once the test budget of cxgDebugFailAllocs is spent.
cudaError_t dev_malloc(void **p, size_t n);
cudaError_t dev_malloc_async(void **p, size_t n, cudaStream_t s);
cudaError_t dev_free(void *p);
cudaError_t dev_free_async(void *p, cudaStream_t s);
cudaError_t host_alloc(void **p, size_t n);

// Thread-local error message.
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t err, const char *what);

// Stream capture and device-wide synchronisation exclude each other: a
// call that synchronises the device (cudaFree, cudaFreeHost,
// cudaDeviceSynchronize) on one thread while another thread captures a
// stream invalidates that capture.  Captures hold this lock from begin to
// end; the library's frees and device synchronisations go through
// dev_free, host_free and device_sync, which take it.
std::mutex &capture_gate();
cudaError_t host_free(void *p);
cudaError_t device_sync();

// lnL of the chain at heat 1 after the work queued on an MC3 handle (one
// synchronisation of its stream, two copies); -inf if no chain is cold.
int mc3_cold_lnl(cxgMc3 *h, double *out);

#define CXG_CUDA(call)                                         \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cxg::cuda_fail(e_, #call); \
    } while (0)

#define CXG_CHECK_LAUNCH(what)                                 \
    do {                                                       \
        cudaError_t e_ = cudaGetLastError();                   \
        if (e_ != cudaSuccess) return cxg::cuda_fail(e_, what);  \
    } while (0)

// Kernel launchers (cxg_kernels.cu).
cudaError_t launch_pmat(const PmatArgs &a, cudaStream_t s);
cudaError_t launch_pmat_batch(const PmatArgs *jobs, const uint32_t *prefix,
                              uint32_t njobs, uint32_t total, cudaStream_t s);
// `lanes` 2: the op-lane walker (the plan's records come in steps of two).
// `pdl`: launch as a programmatic dependent of the P kernel launched just
// before it on `s` (the walker stages its leaves while the P kernel runs).
cudaError_t launch_plan(int precision, const PlanArgs &a, cudaStream_t s,
                        unsigned lanes = 1, bool pdl = false);
cudaError_t launch_qdecomp(const double *rtri, const double *pi, double *out,
                           cudaStream_t s);
unsigned plan_blocks(unsigned ppad, unsigned tile);
// try_wait attempts of the walkers' record waits on the current device
// (0: give up without waiting).
cudaError_t set_spin_limit(uint32_t limit);

}  // namespace cxg
