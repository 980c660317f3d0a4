// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "cxlik_gpu.h"

namespace cxg {

// Patterns are padded to a multiple of this on the device, so that every
// plane of a CL buffer starts on a 512-byte boundary.
constexpr unsigned kPatternQuantum = 128;
// Threads per CTA of the plan walkers.
constexpr unsigned kBlock = 128;
// Largest number of active mixture components held in registers.
constexpr unsigned kMaxComps = 8;
// Largest node degree handled in one op (children per parent).
constexpr unsigned kMaxChildren = 16;

inline unsigned pad_patterns(unsigned p) {
    return (p + kPatternQuantum - 1) / kPatternQuantum * kPatternQuantum;
}

// One child of an op.  `data` is a CL buffer ([K][4][ppad] of the op's
// precision) or, for a leaf, uint8 masks [ppad]; `scaler` is the child's
// per-pattern log scale (FP64) or power-of-two exponent (FP32), null for a
// leaf.  `pm` indexes the child's block of P matrices / leaf tables.
struct DevChild {
    const void *data;
    const void *scaler;
    uint32_t leaf;
    uint32_t pm;
};

// One node update: the parent CL and the range of its children.
struct DevOp {
    void *data;
    void *scaler;
    uint32_t child0;
    uint32_t nchild;
};

// Per-call constants of a plan execution.
struct PlanArgs {
    const DevOp *ops;
    const DevChild *children;
    uint32_t nops;
    uint32_t kact;        // active components (weightScaled != 0)
    uint32_t npat;        // patterns (mschars)
    uint32_t ppad;        // padded pattern stride
    const void *pm;       // [nchild][kact][16] P matrices (double or float)
    const void *ltab;     // [nchild][16 masks][kact][4] leaf messages
    const double *pn;     // [kact][4] pi_i * weightScaled (root weights)
    const void *root;     // root CL buffer
    const void *rootsc;   // root scaler
    const uint32_t *freqs;// [npat] pattern weights (charFreqs + cbase)
    double *site;         // [npat] site lnL out (may be null)
    double *partial;      // [nblocks][2] compensated partial sums
    uint32_t *ninf;       // count of -inf sites
    unsigned *ticket;     // last-block counter
    double *total;        // [2] final (sum, compensation)
};

// Inputs of the P-matrix kernel: one row per (child, active comp).
struct PmatArgs {
    uint32_t nchild;
    uint32_t kact;
    const double *edge_len;    // [nchild]
    const uint32_t *leafflag;  // [nchild]
    const double *cmult;       // [kact]
    const double *rmult;       // [kact]
    const int32_t *model;      // [kact] model index of each active comp
    const double *cube;        // [nmodels][64]
    const double *eig;         // [nmodels][4]
    double wnorm;
    double *pm64;              // [nchild][kact][16]
    float *pm32;
    double *ltab64;            // [nchild][16][kact][4]
    float *ltab32;
};

// Thread-local error message.
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t err, const char *what);

// Kernel launchers (cxg_kernels.cu).
cudaError_t launch_pmat(const PmatArgs &a, cudaStream_t s);
cudaError_t launch_plan(int precision, const PlanArgs &a, cudaStream_t s);
cudaError_t launch_qdecomp(const double *rtri, const double *pi, double *out,
                           cudaStream_t s);
unsigned plan_blocks(unsigned ppad);

}  // namespace cxg
