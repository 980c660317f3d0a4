/*
 * cxlik_gpu.h -- C ABI of the GB300 pruning-likelihood library
 * (crux_gb300/_lib/libcxlik_gpu.so).
 *
 * Part 1 is the drop-in boundary: the structures and the three entry points
 * that Crux's Lik object (pkg/Crux/Tree/Lik.pyx) fills and calls.  Their
 * layout and meaning are those of lib/Crux/Tree/CxLik.h; a caller built
 * against that header links against this library unchanged.
 *
 * Part 2 holds the additional cxg* entry points: device-resident leaf data,
 * cache release, an lnL-only execute, the FP32-scaled form, the batched
 * persistent kernel, on-device MC3 and the serving loop.  They have no
 * counterpart in the reference; each says what it adds.
 *
 * Error convention: CxLikQDecomp returns true on error (as the reference);
 * every cxg* function returns 0 on success and a negative CXG_E* code on
 * error; cxgLastError() gives a message for the most recent failure,
 * including failures inside the void CxLikExecute.
 */
#ifndef CXLIK_GPU_H
#define CXLIK_GPU_H

#include <stdbool.h>
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Part 1: drop-in structures (lib/Crux/Tree/CxLik.h:6-273).                 */
/* ------------------------------------------------------------------------ */

typedef struct CxsLikCL CxtLikCL;
typedef struct CxsLikModel CxtLikModel;

/* Conditional-likelihood (CL) cache of one directed half-edge
 * (CxLik.h:9-60).  cLMat holds mschars rows of dim*ncomp doubles for an
 * internal node, or mschars rows of dim doubles (0/1 state indicators) for a
 * leaf.  This library treats the host cLMat/lnScale pointers as identities
 * of device-resident buffers: internal CLs live only on the device and the
 * host buffers are neither read nor written; leaf rows are read once, on
 * first use, unless cxgLikClSetLeafMasks registered them. */
struct CxsLikCL {
    double *cLMat;
    double *lnScale;
    bool valid;
    CxtLikCL *parent;
    unsigned nSibs;
    double edgeLen;
};

/* Mixture component (CxLik.h:64-81). */
typedef struct {
    CxtLikModel *model;
    double weightScaled;
    double cweight;
    double cmult;
} CxtLikComp;

/* Mixture model (CxLik.h:90-139). */
struct CxsLikModel {
    bool decomp;
    double weight;
    double qNorm;
    double rmult;
    unsigned *rclass;
    double *rTri;
    double *piDiag;
    double *piDiagNorm;
    double *qEigVecCube;
    double *qEigVals;
    double alpha;
    bool catMedian;
    bool invar;
    unsigned comp0;
    unsigned clen;
};

/* Step variants (CxLik.h:150-155). */
typedef enum {
    CxeLikStepComputeL = 0,
    CxeLikStepComputeI = 1,
    CxeLikStepMergeL = 2,
    CxeLikStepMergeI = 3
} CxeLikStep;

/* One planned step (CxLik.h:168-174). */
typedef struct {
    CxeLikStep variant;
    unsigned ntrail;
    CxtLikCL *parentCL;
    CxtLikCL *childCL;
    double edgeLen;
} CxtLikStep;

/* The likelihood object (CxLik.h:176-273, built without CxmMpi). */
typedef struct {
    unsigned polarity;
    unsigned dim;
    unsigned rlen;
    unsigned cbase;
    unsigned nchars;
    unsigned mschars;
    unsigned npad;
    unsigned *charFreqs;
    unsigned stripeWidth;
    unsigned nstripes;
    bool invalidate;
    bool resize;
    bool reweight;
    double wNorm;
    CxtLikModel **models;
    unsigned modelsLen;
    unsigned modelsMax;
    CxtLikComp *comps;
    unsigned compsLen;
    unsigned compsMax;
    CxtLikCL *rootCLC;
    double *siteLnL;
    double *stripeLnL;
    CxtLikStep *steps;
    unsigned stepsLen;
    unsigned stepsMax;
} CxtLik;

/* Replaces CxLikQDecomp (CxLik.h:279-281; definition CxLik.c:177-250, whose
 * argument order -- qNorm before the cube -- is the one callers use,
 * Lik.pyx:472-474).  Normalises PiDiag into PiDiagNorm, builds
 * Q = R*Pi with zero row sums, sets qNorm = 1/(2*sum_{i<j} R_ij pi_i pi_j),
 * and writes qEigVecCube[i][j][k] = V[i][k]*Vinv[k][j] and the n real
 * eigenvalues.  The decomposition runs in FP64 on the GPU (symmetrised
 * Jacobi; Q of a reversible model is similar to a symmetric matrix).
 * Returns true on error (n != 4, non-positive frequency, no GPU). */
bool CxLikQDecomp(int n, double *RTri, double *PiDiag, double *PiDiagNorm,
                  double *qNorm, double *qEigVecCube, double *qEigVals);

/* Replaces CxLikPt (CxLik.h:282-283; CxLik.c:258-292):
 * P[i*n+j] = max(0, sum_k cube[i][j][k]*exp(eigVals[k]*v)).  Host FP64. */
void CxLikPt(int n, double *P, double *qEigVecCube, double *qEigVals,
             double v);

/* Replaces CxLikExecute (CxLik.h:284-285; CxLik.c:914-968).  Runs the
 * lik->steps plan on the GPU in FP64 with the reference's per-pattern
 * scaler, then writes siteLnL[cbase .. cbase+mschars) and
 * stripeLnL[0 .. nstripes).  Failures leave a message in cxgLastError(). */
void CxLikExecute(CxtLik *lik);

/* ------------------------------------------------------------------------ */
/* Part 2: additions (no counterpart in the reference).                      */
/* ------------------------------------------------------------------------ */

enum {
    CXG_OK = 0,
    CXG_EINVAL = -1,   /* bad argument or unsupported shape */
    CXG_ENOMEM = -2,   /* device or host allocation failed */
    CXG_ECUDA = -3,    /* CUDA runtime error */
    CXG_ETIMEOUT = -4, /* a bounded device wait gave up */
    CXG_EBUSY = -5     /* admission refused (serving loop) */
};

/* Precision of a plan execution. */
enum {
    CXG_FP64 = 0,      /* plain: FP64 CLVs, the reference's scaler */
    CXG_FP32 = 1       /* FP32 CLVs, per-pattern power-of-two exponents */
};

/* Message describing the most recent failure on the calling thread. */
const char *cxgLastError(void);

/* Library version and build facts: writes "cxlik_gpu <ver> sm_103a ..." */
int cxgInfo(char *buf, size_t len);

/* Register leaf CL `cl` (identified by cl->cLMat) with n per-pattern state
 * masks (bit j set = state j allowed; 0 is treated as "any", as
 * Lik.pyx:1469-1470).  Replaces the host upload of mschars*4 doubles. */
int cxgLikClSetLeafMasks(const CxtLikCL *cl, const uint8_t *masks,
                         unsigned n);

/* Release the device buffers behind a host CL identity.  Call when the
 * host cLMat is freed (CL.flush / CL.__dealloc__ in Lik.pyx:47-53, 98-107),
 * so that a later allocation at the same address is not mistaken for it. */
int cxgLikClForget(const double *cLMat);

/* Release every device buffer and cached plan. */
int cxgLikReset(void);

/* Register a Lik's pattern weights (charFreqs + cbase, n = mschars): they
 * are uploaded now and the caller promises not to change them while
 * registered, so plans skip comparing them with the kept copy.  No
 * counterpart in the reference (Lik.pyx:314 borrows Alignment.freqs, which
 * does not change after compaction).  Unregistered weights are compared on
 * every call and uploaded again when they differ.  Forget them before the
 * host array is freed or changed. */
int cxgLikSetPatternWeights(const unsigned *freqs, unsigned n);
int cxgLikForgetPatternWeights(const unsigned *freqs, unsigned n);

/* Execute lik's plan at the given precision; write the compensated FP64
 * sum of site lnLs to *lnL (one 8-byte device-to-host copy).  If siteLnL is
 * non-NULL also fill it (mschars doubles, pad patterns included). */
int cxgLikExecuteLnL(CxtLik *lik, int precision, double *lnL,
                     double *siteLnL);

/* Bytes copied host->device and device->host by the most recent
 * cxgLikExecuteLnL / CxLikExecute (program upload; result read-back). */
int cxgLikLastIo(size_t *h2d, size_t *d2h);

/* Device memory currently held for CL buffers, in bytes. */
int cxgLikDeviceBytes(size_t *bytes);

/* A translated plan: lik->steps turned into a device program once and run
 * any number of times (e.g. to time it, or to re-evaluate after changing
 * nothing but branch lengths in the same CxtLikStep array -- call
 * cxgPlanCreate again after any change).  The CL buffers the plan
 * references must stay registered while it exists. */
typedef struct cxgPlan cxgPlan;
int cxgPlanCreate(CxtLik *lik, int precision, cxgPlan **plan);
/* Run once and wait; lnL as cxgLikExecuteLnL. */
int cxgPlanRun(cxgPlan *plan, double *lnL, double *siteLnL);
/* Run `iters` times back to back on the device (no host sync between runs);
 * report the mean wall time per run and the mean plan-walker kernel time,
 * both from CUDA events on the library's stream, and the last lnL. */
int cxgPlanTime(cxgPlan *plan, int iters, double *ms_per_run,
                double *plan_kernel_ms, double *lnL);
/* Pattern-node updates per run, algorithmic bytes of one plan-walker
 * launch, node updates (ops) and kernels launched per run. */
int cxgPlanInfo(const cxgPlan *plan, double *updates, double *alg_bytes,
                unsigned *nops, unsigned *kernels_per_run);
int cxgPlanDestroy(cxgPlan *plan);
/* Launch shape chosen for a plan: patterns per CTA, threads per pattern,
 * patterns per thread, shared-memory stack slots, distinct leaves. */
int cxgPlanShape(const cxgPlan *plan, unsigned *tile, unsigned *threads_per_pattern,
                 unsigned *patterns_per_thread, unsigned *nslot, unsigned *nleaf);
/* Op lanes the plan's walker runs with (cxgTuneLanes). */
int cxgPlanLanes(const cxgPlan *plan, unsigned *lanes);

/* The step planner of Lik._planRecurse / Lik._plan (Lik.pyx:1427-1601) run
 * natively over one rooted traversal of a tree, flattened once by the host
 * mirror.  Visits are in the planner's post-order and the root CL is the
 * last.  Visit v's CL is cl[v], its parent is visit up[v] (-1 for the root),
 * its nSibs and edge length are nsibs[v] and lens[edge[v]] (edge -1 means a
 * length of 0), and its children are kid0[v] .. kid0[v]+nkids[v]-1 (none for
 * a leaf).  A child names the CL a step reads (kid_cl), whether it is
 * internal (kid_int: I or L variants) and its edge (kid_edge).  The five
 * mirror arrays hold each visit's valid, struct-valid, parent, nSibs and
 * edgeLen as the caller last saw them; the planner updates them with the
 * CxtLikCL fields it writes. */
typedef struct {
    uint32_t nvis;
    uint32_t nkid;
    CxtLikCL *const *cl;
    const int32_t *up;
    const uint32_t *nsibs;
    const int32_t *edge;
    const uint32_t *kid0;
    const uint32_t *nkids;
    CxtLikCL *const *kid_cl;
    const uint8_t *kid_int;
    const int32_t *kid_edge;
    uint8_t *valid;
    uint8_t *cvalid;
    CxtLikCL **m_parent;
    uint32_t *m_nsibs;
    double *m_elen;
} cxgPlanSnap;

/* Plan one evaluation (no counterpart entry point: the reference plans in
 * Cython, Lik.pyx:1427-1601).  Like the Python planner it marks a CL dirty
 * when its parent, nSibs or edge length changed (or `invalidate` is set),
 * emits the Compute/Merge steps of every dirty internal CL and of the root,
 * writes changed CxtLikCL fields and finally each CL's valid flag.  Steps go
 * to steps[0 .. *nsteps).  The indices of visits whose mirrors changed go to
 * changed[0 .. *nchanged) (room for nvis).  Returns 0; CXG_EINVAL for a
 * malformed snapshot or a full step array; 1 when a step would carry a
 * negative branch length, with the state as far as the planner had come
 * (the Python planner raises ValueError at the same point). */
int cxgPlanSnapRun(const cxgPlanSnap *snap, const double *lens, int invalidate,
                   CxtLikStep *steps, uint32_t cap, uint32_t *nsteps,
                   uint32_t *changed, uint32_t *nchanged);

/* A batch: the plans of many likelihoods (trees, alignments, models; all
 * with the same number of active components) run by one persistent launch
 * that walks (job, pattern-tile) items, longest jobs first; one run (P
 * matrices, walker, result copy) is captured once as a CUDA graph and
 * replayed.  CXG_BATCH_PER_NODE instead issues one walker launch per node
 * update without the shared-memory stack -- the unfused comparison. */
typedef struct cxgBatch cxgBatch;
enum { CXG_BATCH_PER_NODE = 1 };
int cxgBatchCreate(CxtLik *const *liks, unsigned n, int precision,
                   unsigned flags, cxgBatch **batch);
int cxgBatchRun(cxgBatch *batch, double *lnLs);
/* Mean time per run over `iters` runs (graph launches back to back) and
 * the mean event-timed walker time. */
int cxgBatchTime(cxgBatch *batch, int iters, double *ms_per_run,
                 double *walk_ms);
int cxgBatchInfo(const cxgBatch *batch, double *updates, double *alg_bytes,
                 unsigned *nitems, unsigned *grid,
                 unsigned long long *launches_per_run);
int cxgBatchDestroy(cxgBatch *batch);

/* On-device MC3 (no counterpart entry point in the reference; the
 * reference runs its chains on the host, pkg/Crux/Mc3/Chain.pyx).  All
 * chains share one alignment; each keeps its tree, model, lnL, heat and CLs
 * in HBM.  Nodes 0..ntaxa-1 are the leaves (in mask order), the tree is
 * binary and rooted at internal node `root` (degree 3). */
typedef struct {
    unsigned ntaxa;
    unsigned npat;
    const uint8_t *masks;          /* [ntaxa][npat] state masks, 0 = any */
    const uint32_t *freqs_pattern; /* [npat] pattern weights */
    const int32_t *parent;         /* [2*ntaxa-2], -1 at the root */
    const double *len;             /* [2*ntaxa-2] length of edge to parent */
    unsigned root;
    double rates[6];    /* exchangeabilities AC AG AT CG CT GT */
    double freqs[4];    /* base frequencies */
    double alpha;       /* Gamma shape (ignored when ncat == 1) */
    unsigned ncat;      /* Gamma categories, 1..8 */
    unsigned nchains;
    double heat_delta;  /* chain i runs at heat 1/(1 + i*heat_delta) */
    unsigned swap_stride;
    unsigned long long seed;
    double move_weight[17]; /* branch length, NNI, rates (Dirichlet over
                               the class rates), alpha, base frequencies,
                               SPR, eTBR, +I weights, Gamma on/off jump,
                               equal/estimated frequency jump, +I off/on
                               jump, rate-class merge/split jump, one
                               class rate's multiplier, mixture weight,
                               mixture rate multiplier, mixture member
                               add/remove jump, polytomy jump (an
                               internal edge contracted or restored) */
    double brlen_lambda, brlen_prior;
    double rate_conc;       /* Dirichlet concentration of rate moves */
    double freq_conc;       /* Dirichlet concentration of frequency moves */
    double etbr_pext;       /* eTBR extension probability (the reference's
                               etbrPExt, 0.8), in [0, 1] */
    double alpha_lambda, alpha_prior;
    double pinv;            /* +I weight (0: no +I component); the
                               variable part starts at 1 - pinv */
    double invar_lambda;    /* multiplier of +I weight moves */
    double invar_prior;     /* the reference's invarPrior (0.5): Exp priors
                               of rate 1 - invarPrior on wVar and
                               invarPrior on wInvar */
    double gamma_jump_prior; /* the reference's rateShapeInvJumpPrior (1):
                               prior odds of Gamma off to on */
    double freq_jump_prior;  /* its freqJumpPrior (1): prior odds of equal
                               to estimated base frequencies */
    int precision;          /* CXG_FP32 or CXG_FP64 */
    unsigned graph_gens;    /* generations per captured graph (0: 16) */
    unsigned long long trace_cap;  /* cold-chain lnL trace length */
    double invar_jump_prior; /* the reference's invarJumpPrior (1): prior
                               odds of +I off to on */
    int rclass[6];          /* rate classes of the exchangeabilities, a
                               restricted growth string ({0,1,2,3,4,5}:
                               GTR); rates of one class must be equal */
    double rate_jump_prior; /* the reference's rateJumpPrior (1): prior
                               odds of k-1 to k rate classes */
    double rate_lambda;     /* class-rate multiplier (2 ln 1.6) */
    unsigned max_models;    /* mixture members a chain may hold, 1..4 (0:
                               1); the walker carries max_models x (ncat
                               + +I) components, at most 8 */
    double mixture_jump_prior; /* the reference's mixtureJumpPrior (1/3):
                               k + 1 members have prior odds
                               1 - mixture_jump_prior to k */
    double weight_lambda, rmult_lambda; /* mixture weight and rate
                               multiplier moves (2 ln 1.6) */
    double polytomy_jump_prior; /* the reference's polytomyJumpPrior (1):
                               prior odds of one more contracted edge */
} cxgMc3Config;
/* One mixture member of a chain (alpha is INFINITY with Gamma off). */
typedef struct {
    double rates[6], freqs[4], alpha, wvar, winvar, weight, rmult;
    int rclass[6], nrates, freqs_est;
} cxgMc3ModelState;
/* Calls on one handle are serialised; separate handles (each with its own
 * stream, graph and buffers) may be driven from separate threads at once. */
typedef struct cxgMc3 cxgMc3;
/* Build the chains and run generation 0 (a full evaluation). */
int cxgMc3Create(const cxgMc3Config *cfg, cxgMc3 **mc3);
/* Advance every chain `ngen` generations (one move each, then a heat-swap
 * attempt every swap_stride); *seconds = device time. */
int cxgMc3Run(cxgMc3 *mc3, unsigned long long ngen, double *seconds);
/* Current state of one chain (tree in the same node numbering; the model
 * parameters are its first mixture member's). */
int cxgMc3Chain(cxgMc3 *mc3, unsigned chain, double *lnL, double *heat,
                int32_t *parent, double *len, double *rates, double *freqs,
                double *alpha);
/* Weights (wVar, wInvar) of one chain's first mixture member. */
int cxgMc3ChainWeights(cxgMc3 *mc3, unsigned chain, double *wvar, double *winvar);
/* Contracted edges of one chain's tree: out[v] = 1 where the edge above
 * node v has length 0 and stands for a polytomy (polytomy jumps). */
int cxgMc3ChainCollapsed(cxgMc3 *mc3, unsigned chain, uint8_t *out);
/* Member `model` of one chain's mixture, and the member count. */
int cxgMc3ChainModel(cxgMc3 *mc3, unsigned chain, unsigned model,
                     unsigned *nmodels, cxgMc3ModelState *out);
/* Checkpoint and resume: a chain's tree (rooted at the run's root), heat
 * and mixture members as cxgMc3Chain / cxgMc3ChainModel read them, and the
 * counts of cxgMc3Stats, go into a run built with the same configuration;
 * cxgMc3Resume then recomputes every chain's CLs and lnL and continues at
 * `generation`, drawing what an uninterrupted run draws there. */
int cxgMc3SetChain(cxgMc3 *mc3, unsigned chain, const int32_t *parent,
                   const double *len, const uint8_t *collapsed, double heat,
                   unsigned nmodels, const cxgMc3ModelState *models);
int cxgMc3SetCounts(cxgMc3 *mc3, const unsigned *accepts, const unsigned *rejects,
                    const unsigned *swaps);
int cxgMc3Resume(cxgMc3 *mc3, unsigned long long generation);
/* Accept/reject counts [chain][move] (17 moves, in move_weight order),
 * swaps [chain], generation count. */
int cxgMc3Stats(cxgMc3 *mc3, unsigned *accepts, unsigned *rejects,
                unsigned *swaps, unsigned long long *gen);
/* Cold-chain lnL after each generation 0..n-1. */
int cxgMc3Trace(cxgMc3 *mc3, double *out, unsigned long long n);
int cxgMc3Destroy(cxgMc3 *mc3);

/* Serving loop (no counterpart in the reference).  Requests arrive with
 * their own patterns, tree and model; a worker thread admits them while
 * their device bytes fit the HBM budget, prepares them (model built on the
 * GPU) and runs every prepared likelihood request in the next persistent
 * walker launch, so requests that arrive while others run join the next
 * batch.  MC3-step requests advance on-device chains (kept across requests
 * when `session` is non-zero).  Latencies are measured submit-to-done. */
typedef struct cxgServer cxgServer;
enum { CXG_REQ_LNL = 0, CXG_REQ_MC3 = 1 };
typedef struct {
    unsigned max_active;             /* likelihood jobs admitted at once (0: 256) */
    unsigned long long hbm_budget;   /* device bytes the server may hold (0: 80% free) */
    int precision;                   /* CXG_FP32 or CXG_FP64 */
} cxgServerConfig;
typedef struct {
    int kind;                        /* CXG_REQ_LNL or CXG_REQ_MC3 */
    unsigned ntaxa, npat;
    const uint8_t *masks;            /* [ntaxa][npat] state masks, 0 = any */
    const uint32_t *pattern_freqs;   /* [npat] */
    const int32_t *parent;           /* [2*ntaxa-2], -1 at the root */
    const double *len;               /* [2*ntaxa-2] */
    unsigned root;                   /* internal node of degree 3 */
    double rates[6], freqs[4], alpha;
    unsigned ncat;                   /* Gamma categories (1..8) */
    double pinv;                     /* invariant-site weight (0: no +I) */
    unsigned mc3_gens, mc3_chains;   /* MC3 requests (0: 10 gens, 4 chains) */
    double mc3_heat_delta;
    unsigned long long seed;
    unsigned long long session;      /* MC3: keep chains under this id (0: none) */
    unsigned long long dataset;      /* non-zero: patterns of a dataset added by
                                        cxgServerAddDataset (masks and
                                        pattern_freqs are then ignored) */
} cxgRequest;
typedef struct {
    unsigned long long completed, batches, max_batch;
    unsigned long long bytes_peak, bytes_budget;
    double p50_ms, p99_ms, max_ms, wall_s, updates;
    unsigned long long deferrals;   /* lnL requests put back in the queue
                                       because their memory could not be had
                                       until batches in flight finished */
} cxgServerStatsT;
int cxgServerCreate(const cxgServerConfig *cfg, cxgServer **server);
/* Copies the request; returns at once with a ticket.  Thread-safe. */
int cxgServerSubmit(cxgServer *server, const cxgRequest *req,
                    unsigned long long *ticket);
/* Wait up to timeout_s for a ticket; lnL (cold chain for MC3) and latency. */
int cxgServerWait(cxgServer *server, unsigned long long ticket,
                  double timeout_s, double *lnL, double *latency_ms);
/* Keep a pattern set resident on the device under `id` (non-zero) for the
 * requests that name it; its bytes count against the HBM budget until
 * cxgServerDropDataset (freed once no admitted request uses it). */
int cxgServerAddDataset(cxgServer *server, unsigned long long id,
                        unsigned ntaxa, unsigned npat, const uint8_t *masks,
                        const uint32_t *pattern_freqs);
int cxgServerDropDataset(cxgServer *server, unsigned long long id);
/* The same from a raw alignment rows [ntaxa][nsites] (character codes):
 * the server compacts it on the device (as cxgCompact: canon, val and
 * any_mask of the character type) and keeps the patterns resident without
 * a host round trip; *npat receives the pattern count requests must use. */
int cxgServerAddDatasetRaw(cxgServer *server, unsigned long long id,
                           unsigned ntaxa, unsigned nsites, const uint8_t *rows,
                           const uint8_t *canon, const uint8_t *val,
                           uint8_t any_mask, unsigned *npat);
int cxgServerStats(cxgServer *server, cxgServerStatsT *stats);
int cxgServerResetStats(cxgServer *server);
int cxgServerDestroy(cxgServer *server);

/* Pattern compression on the device (Alignment.compact,
 * pkg/Crux/CTMatrix.pyx:949-1031, after canonize :856-887): the sorted
 * unique columns of rows [ntaxa][nsites] (character codes) with summed
 * frequencies (freqs NULL: 1 per site), bit-exact with the host algorithm:
 * characters map through canon[256], columns order bytewise, identical
 * columns merge.  Writes rows_out [ntaxa][npat] (canonical codes; may be
 * NULL), freqs_out [npat], and when masks_out is given the leaf-tip
 * encoding masks_out [ntaxa][npat] = val[code] & 15, 0 -> any_mask
 * (Lik.pyx:1466-1475).  Output arrays need room for nsites patterns. */
int cxgCompact(const uint8_t *rows, unsigned ntaxa, unsigned nsites,
               const uint32_t *freqs, const uint8_t *canon, const uint8_t *val,
               uint8_t any_mask, uint8_t *rows_out, uint32_t *freqs_out,
               uint8_t *masks_out, unsigned *npat);

/* Launch shape of the plan walker for plans translated from now on:
 * patterns per CTA (32, 64 or 128), threads per pattern (1, 2 or 4: the
 * FP32 form splits a pattern's components over that many threads when the
 * count divides them; tile x threads <= 256), patterns per thread (1 or 2:
 * the FP32 form with one thread per pattern and <= 5 components can give a
 * thread two patterns; tile >= 64) and the shared-memory budget of its CL
 * stack (bytes, <= 200 KiB).  Every shape gives the same bits.  Chosen by
 * the autotuner (crux_gb300.tune). */
int cxgTune(unsigned tile, unsigned threads_per_pattern,
            unsigned patterns_per_thread, size_t smem_budget);
int cxgTuneGet(unsigned *tile, unsigned *threads_per_pattern,
               unsigned *patterns_per_thread, size_t *smem_budget);
/* Op lanes of the single-plan walker (cxgLikExecuteLnL, CxLikExecute,
 * cxgPlanCreate), 1 or 2.  With 2, plans of the FP32 form that stage their
 * leaves, with one thread and one pattern per thread and <= 5 components,
 * run two mutually independent node updates per step on two groups of
 * threads over the same patterns; other plans keep one lane.  Same bits. */
int cxgTuneLanes(unsigned lanes);
int cxgTuneLanesGet(unsigned *lanes);

/* Failure paths, for tests (no counterpart in the reference).
 * cxgDebugSetSpinLimit: mbarrier.try_wait attempts the plan walkers make
 * per op-record wait before giving up (the default is 2^26; 0 gives up at
 * once).  A walk that gives up drains its copies in flight, sets the run's
 * error word and the call returns CXG_ETIMEOUT; the CLs it was computing
 * count as not computed.  Waits for the device to be idle first; *previous
 * (optional) receives the bound it replaces.
 * cxgDebugFailAllocs: let `after` more device or pinned-host allocations
 * of the library succeed, then fail every one as an out-of-memory
 * (CXG_ENOMEM) without calling CUDA; negative: off. */
int cxgDebugSetSpinLimit(unsigned limit, unsigned *previous);
int cxgDebugFailAllocs(long long after);
/* cxgDebugCanaries: give every later device allocation of the library a
 * 256-byte canary after its end (also on when CXG_DEBUG_CANARY is set in
 * the environment).  cxgDebugCheckCanaries: wait for the device, read every
 * live allocation's canary back, and count those changed since (with any a
 * synchronous free found changed). */
int cxgDebugCanaries(int on);
int cxgDebugCheckCanaries(unsigned long long *checked, unsigned long long *bad);
/* The check itself: a 1000-byte allocation whose canary a host memset
 * changes must read as changed (*detected = 1).  Canaries must be on. */
int cxgDebugCanarySelfTest(int *detected);

/* No counterpart in the reference.  Evaluate lik's plan without allocating
 * anything, for callers that cannot call cudaMalloc.  Such a caller may
 * own the device heap through its own pool or allocator, or may be on a
 * latency-critical path where cudaMalloc/cudaFree could synchronise the
 * device.  Every memory the computation touches is the caller's:
 *   - each CxtLikCL in lik->steps and lik->rootCLC holds DEVICE pointers:
 *     internal CL: cLMat -> kact*4*ceil128(mschars) elements of the
 *     precision (double or float) laid out [kact][U][ppad] in 16-byte
 *     units, lnScale -> ppad scalers (double for CXG_FP64, int32 for
 *     CXG_FP32; size the buffer for 8 bytes per pattern); leaf CL: cLMat
 *     -> ppad uint8 state masks (pad patterns set to 15), lnScale unused;
 *     every cLMat 16-byte aligned, as cudaMalloc returns;
 *   - dFreqs: mschars uint32 pattern weights on the device;
 *   - dSiteLnL: optional device output of mschars site lnLs (NULL: none);
 *   - stream: the caller's cudaStream_t (NULL: the default stream).
 * Scratch is a fixed 4 MiB device array in the library (every GPU that
 * loads the library holds it until exit); limits: <= 1024 node updates,
 * <= 2048 children, <= 2^20 patterns, <= 8 active components.  The first
 * call on a device looks up that array's address: make it before any
 * stream capture.  With CUDA's lazy module loading, the first call of each
 * precision on a device also loads the library's kernels, which the CUDA driver
 * may allocate for: make one call of each precision as a warm-up outside
 * the region where nothing may allocate.  Calls share the array; calls
 * that overlap on the GPU race.  Returns after the lnL has been copied
 * back. */
int cxgLikExecuteNoAlloc(const CxtLik *lik, int precision,
                         const uint32_t *dFreqs, double *dSiteLnL,
                         void *stream, double *lnL);

#ifdef __cplusplus
}
#endif

#endif /* CXLIK_GPU_H */
