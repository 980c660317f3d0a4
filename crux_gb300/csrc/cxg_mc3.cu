// On-device Metropolis-coupled MCMC (MC3) over the pruning likelihood.
//
// The reference runs each chain on the host: a proposal mutates the tree or
// the model, Lik.lnL recomputes the dirty path, and a Metropolis test in
// FP64 accepts or rejects it; chains swap heats every swapStride steps
// (pkg/Crux/Mc3/Chain.pyx:438-476 brlenPropose, :320-377
// rateShapeInvPropose, :1816-1911 advance0/advance1; heats
// 1/(1 + ind * heatDelta), :51).  Here all chains live in HBM and one
// generation is four kernels, captured together into a CUDA graph:
//
//   mc3_propose  one block per chain: flip in the CL buffers of the last
//                accepted move, draw the move (Philox), apply it to the
//                chain's tree or to the spare model slot, list the dirty
//                internal nodes bottom-up, and write their op records.
//                Dirty CLs go to each node's spare CL buffer, so a rejected
//                move costs no restore.
//   mc3_pmat     P matrices of every child edge of every chain's ops.
//   walk_batch   the batched plan walker over (chain, pattern tile) items.
//   mc3_accept   FP64 Metropolis per chain, then the heat swap; rejected
//                tree moves are undone.
//
// Moves (weights set by the caller): branch-length multiplier (as the
// reference: m = exp(lambda (u - 1/2)), Exp(brlenPrior) prior, Hastings
// ln m); NNI across a random internal edge (symmetric); GTR
// exchangeabilities and base frequencies, each from a Dirichlet centred on
// the current values (flat Dirichlet prior, Hastings from the two
// Dirichlet densities); the inverse Gamma shape multiplier of the
// reference (rateShapeInvPropose, Exp(1) prior on 1/alpha); SPR: prune a
// subtree whose parent p is not the root (p's two edges merge), regraft p
// on a uniform edge outside the subtree, split at a uniform point.  SPR
// keeps the tree length (prior ratio 1 under iid exponential lengths); the
// pruned tree and so the edge count are the same both ways, and the
// Jacobian of (l_p, l_b, l_x, u) -> (l_b + l_p, u l_x, (1 - u) l_x,
// l_p / (l_p + l_b)) gives the Hastings ratio l_x / (l_b + l_p).
// Extending TBR (etbrPropose, Chain.pyx:478-819): each end of a uniform
// edge eA moves its node along a random path, extended with probability
// etbr_pext per step, into the path's last edge; the lengths of eA and of
// the first edge of each path get multipliers.  A chain's tree has two
// buffers: an eTBR move writes the re-rooted result into the spare one,
// which an accepted move makes current.  Reversible jumps: Gamma on/off,
// equal/estimated frequencies, +I off/on, rate classes merged/split,
// mixture members added/removed, with the mixture weight and rate
// multiplier moves, and polytomies (an internal edge contracted or
// restored) (Chain.pyx:72-141, 200-266, 821-1814); each model move
// changes one uniform member of a chain's mixture.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "cxg_devmath.cuh"
#include "cxg_device.cuh"
#include "cxg_internal.h"

namespace cxg {

enum {
    MV_BRLEN = 0, MV_NNI = 1, MV_RATES = 2, MV_ALPHA = 3, MV_FREQS = 4, MV_SPR = 5,
    MV_ETBR = 6, MV_INVAR = 7, MV_GAMMAJ = 8, MV_FREQJ = 9, MV_INVARJ = 10,
    MV_RATEJ = 11, MV_RATE1 = 12, MV_WEIGHT = 13, MV_RMULT = 14, MV_MIXJ = 15,
    MV_POLYJ = 16, MV_INIT = 17
};
constexpr int kMoves = 17;
// Moves that change the model (the spare model slot).
constexpr uint32_t kModelMoves =
    (1u << MV_RATES) | (1u << MV_ALPHA) | (1u << MV_FREQS) | (1u << MV_INVAR) |
    (1u << MV_GAMMAJ) | (1u << MV_FREQJ) | (1u << MV_INVARJ) | (1u << MV_RATEJ) |
    (1u << MV_RATE1) | (1u << MV_WEIGHT) | (1u << MV_RMULT) | (1u << MV_MIXJ);
// Most models in a chain's mixture.
constexpr int kMaxModels = 4;

// One model of a chain's mixture (a CxtLikModel with its parameters).
struct Mc3Sub {
    // rates: the six exchangeabilities; those of one rate class (rclass, a
    // restricted growth string with nrates classes) are equal.
    double rates[6], freqs[4], alpha;
    int32_t rclass[6], nrates;
    double wvar, winvar;  // weights of the variable and +I parts
    // 0: Gamma rates off (the reference's alpha = INFINITY: all variable
    // weight on the first category, rate 1); 0: equal base frequencies.
    int32_t gamma_on, freqs_est;
    double weight, rmult;       // mixture weight and rate multiplier
    double gcat[kMaxComps];     // Gamma category rates (Gamma on)
};

// A chain's model: nmodels mixture members in slots 0..nmodels-1.  The
// walker's components are model-major, kper = ncat (+1 with +I) per slot
// for mmax slots; the components of unused slots carry weight 0 and model
// 0's matrices, so their rows stay finite.
struct Mc3Model {
    Mc3Sub q[kMaxModels];
    int32_t nmodels;
    double pinorm[kMaxModels * 4], qnorm[kMaxModels];
    double cube[kMaxModels * 64], eig[kMaxModels * 4];
    double cmult[kMaxComps], rmult[kMaxComps];
    int32_t midx[kMaxComps];
    double wnorm;
    double pn[kMaxComps * 4];
    int32_t ok;
};

struct Mc3Prop {
    int32_t type, node, a, c;
    double oldlen, lnPrior, lnHast;
    int32_t model_changed, ndirty;
    // Set by the accept kernel; the next proposal flips the dirty nodes'
    // CL buffers in when it is set.
    int32_t accepted;
    // SPR undo: subtree s, its parent p, p's old parent g and other child b,
    // target x and its parent xp in the pruned tree; child slots of p in g,
    // of b in p and of x in xp; the old lengths of b, p and x.
    int32_t s, p, g, b, x, xp, jg, jb, jx;
    double lb, lp, lx;
};

struct Mc3Dev {
    uint32_t nchains, ntaxa, nnodes, root, kact, npat, ppad, prec;
    uint32_t ncat, invar;  // kper = ncat Gamma categories (+1 with +I)
    uint32_t kper, mmax;   // components per model; kact = mmax * kper
    uint32_t rstride, M, maxkids, ntiles;
    // Two tree buffers per chain, b = curtree[c] current: buffer b of
    // chain c starts at (b * nchains + c) * nnodes entries.
    int32_t *parent;      // [2][c][nnodes]
    int32_t *child;       // [2][c][nnodes][3]
    double *len;          // [2][c][nnodes]
    // [2][c][nnodes]: the edge above node v is contracted (length 0): its
    // two ends are one node of a multifurcating tree (polytomy jumps).
    uint8_t *coll;
    uint8_t *curtree;     // [c]
    uint8_t *cur;         // [c][nnodes]
    int32_t *dirty;       // [c][M] dirty internal nodes, bottom-up
    // A full walk's op order, children and stack slots, kept per chain
    // while its topology stays: fl_nd[c] ops (0: not kept), the order
    // [c][M], the children prefix [c][M + 1], op and child slots [c][4M].
    int32_t *fl_nd, *fl_dirty;
    uint32_t *fl_kid0;
    int8_t *fl_slot;
    int32_t *stack;       // [c][nnodes] DFS scratch
    void **cl_data;       // [c][M][2]
    void **cl_sc;         // [c][M][2]
    const uint8_t *const *leafmask;  // [ntaxa]
    Mc3Model *model;      // [c][2]
    uint8_t *curmodel;    // [c]
    double *lnL, *heat;   // [c]
    uint64_t seed;
    uint64_t *gen;        // generation counter
    Mc3Prop *prop;        // [c]
    PlanArgs *jobs;       // [c]
    unsigned char *rec;   // [c][M][rstride]
    const uint8_t **lrows;  // [c][M][3] leaf-child mask arrays of each op
    double *kid_len;      // [c][maxkids]
    uint64_t *kid_dst;    // [c][maxkids]
    int32_t *kid_tab;     // [c][maxkids]
    uint32_t *nkids;      // [c]
    double *ltab;         // [c][maxkids][16][kact][4] (FP64 chains)
    char *results;        // [c][32]
    unsigned *counter;
    double wcdf[kMoves];
    double brlen_lambda, brlen_prior, rate_conc, alpha_lambda, alpha_prior;
    double freq_conc, etbr_pext, invar_lambda, invar_prior;
    double gamma_jump_prior, freq_jump_prior, invar_jump_prior;
    double rate_jump_prior, rate_lambda;
    double mix_jump_prior, weight_lambda, rmult_lambda;
    double polytomy_jump_prior;
    uint32_t poly;  // polytomy jumps on (trees may hold contracted edges)
    // Moves with a non-zero weight (bit per MV_*): a new mixture member's
    // parameters are drawn from the prior where a move can change them,
    // else copied from slot 0.
    uint32_t moves_on;
    uint32_t swap_stride;
    uint32_t *acc, *rej;  // [c][kMoves]
    uint32_t *nswap;      // [c]
    double *trace;        // [trace_cap] cold-chain lnL after each generation
    uint64_t trace_cap;
    uint32_t *status;     // nonzero: a model could not be decomposed
    uint32_t nslot_cap;   // shared-memory stack slots of the walker
    uint32_t staged;      // leaves staged per tile (else streamed)
};

// wNorm and the root weights of a mixture whose members' eigensystems and
// category rates are set (Lik.pyx:1603-1665).  Component weights as
// Lik.setWVar / setWInvar leave them within a member: wVar / ncat for each
// Gamma category and wInvar for the +I component (cmult 0), scaled by
// their sum; across members, by weight / (sum of the members' weights).
// wNorm = 1 / sum of weightScaled * rmult / qNorm over components with
// non-zero weight and rate; the +I components stay out of it.
__device__ void mc3_model_weights(Mc3Model &m, unsigned ncat, unsigned invar,
                                  unsigned mmax) {
    const unsigned kper = ncat + (invar ? 1u : 0u);
    double wsum = 0.0;
    for (int mi = 0; mi < m.nmodels; ++mi) wsum += m.q[mi].weight;
    double qmean = 0.0;
    for (unsigned mi = 0; mi < mmax; ++mi) {
        const bool on = (int)mi < m.nmodels;
        const unsigned src = on ? mi : 0u;
        const Mc3Sub &s = m.q[src];
        double cw[kMaxComps], cm[kMaxComps], cwsum = 0.0;
        for (unsigned k = 0; k < ncat; ++k) {
            cw[k] = s.wvar / ncat;
            cm[k] = ncat == 1 ? 1.0 : s.gcat[k];
        }
        if (ncat > 1 && !s.gamma_on) {
            // Lik.setAlpha(INFINITY), Lik.pyx:1264-1273: the first category
            // takes all the variable weight at rate 1, the others weight 0.
            cw[0] = s.wvar;
            cm[0] = 1.0;
            for (unsigned k = 1; k < ncat; ++k) {
                cw[k] = 0.0;
                cm[k] = 0.0;
            }
        }
        if (invar) {
            cw[ncat] = s.winvar;
            cm[ncat] = 0.0;
        }
        for (unsigned k = 0; k < kper; ++k) cwsum += cw[k];
        for (unsigned k = 0; k < kper; ++k) {
            const unsigned c = mi * kper + k;
            const double ws = on ? (s.weight / wsum) * (cw[k] / cwsum) : 0.0;
            m.cmult[c] = cm[k];
            m.rmult[c] = s.rmult;
            m.midx[c] = (int32_t)src;
            if (ws != 0.0 && cm[k] != 0.0) qmean += ws * (s.rmult / m.qnorm[src]);
            for (int i = 0; i < 4; ++i) m.pn[c * 4 + i] = m.pinorm[src * 4 + i] * ws;
        }
    }
    m.wnorm = 1.0 / qmean;
    m.ok = 1;
}

// Parts of a model to derive again: FIN_EIG (rates or frequencies changed),
// FIN_GAMMA (alpha), FIN_WEIGHTS (weights only: +I weights, mixture
// weights and rate multipliers, members added or removed).
enum : unsigned { FIN_EIG = 1, FIN_GAMMA = 2, FIN_ALL = 3, FIN_WEIGHTS = 4 };

// Derived quantities of mixture member `mi`: its Q eigensystem (FP64
// Jacobi on the device) and Gamma category rates, then wNorm and the root
// weights of the whole mixture (Lik.pyx:1603-1665); the parts `what` does
// not name are kept.  One warp: lanes 0..ncat-2 compute the Gamma category
// cuts while lanes 28..31 form the eigensystem; lane 0 finishes.  All 32
// lanes of the warp call it; the result (true: decomposed) is lane 0's.
__device__ bool mc3_model_finish_warp(Mc3Model &m, unsigned ncat, unsigned invar,
                                      unsigned mmax, unsigned what, unsigned mi) {
    __shared__ double s_cut[kMaxComps];
    __shared__ double s_eig[74];
    __shared__ int s_bad;
    Mc3Sub &q = m.q[mi];
    const unsigned lane = threadIdx.x & 31u;
    if (lane == 0) s_bad = 0;
    __syncwarp();
    if ((what & FIN_GAMMA) && ncat > 1 && q.gamma_on && lane < ncat - 1) {
        const double cut = d_gamma_cut(q.alpha, (int)ncat, (int)lane);
        if (cut == -1.0)
            s_bad = 1;
        else
            s_cut[lane] = cut;
    }
    if ((what & FIN_EIG) && lane >= 28) qdecomp4_warp(q.rates, q.freqs, s_eig, 28);
    __syncwarp();
    if ((what & FIN_EIG) && lane == 31) {
        const double *tmp = s_eig;
        if (tmp[73] != 0.0) {
            s_bad = 1;
        } else {
            for (int i = 0; i < 4; ++i) m.pinorm[mi * 4 + i] = tmp[i];
            m.qnorm[mi] = tmp[4];
            for (int i = 0; i < 64; ++i) m.cube[mi * 64 + i] = tmp[5 + i];
            for (int i = 0; i < 4; ++i) m.eig[mi * 4 + i] = tmp[69 + i];
        }
    }
    __syncwarp();
    if (lane != 0) return false;
    if (s_bad) return false;
    if ((what & FIN_GAMMA) && ncat > 1 && q.gamma_on) {
        for (unsigned i = 0; i + 1 < ncat; ++i) q.gcat[i] = s_cut[i];
        d_gamma_rates_from_cuts((int)ncat, q.gcat);
    }
    mc3_model_weights(m, ncat, invar, mmax);
    return true;
}

__global__ void mc3_init_kernel(Mc3Dev d) {
    const unsigned c = blockIdx.x;
    if (c >= d.nchains || threadIdx.x >= 32) return;
    Mc3Model &m = d.model[c * 2 + d.curmodel[c]];
    bool ok = true;
    for (int mi = 0; mi < m.nmodels; ++mi)
        ok &= mc3_model_finish_warp(m, d.ncat, d.invar, d.mmax, FIN_ALL, (unsigned)mi);
    if (threadIdx.x == 0 && !ok) atomicOr(d.status, 1u);
}

// log density of Dirichlet(alpha) at x (both length n).
// Partitions of the six exchangeabilities into k classes, k = 1..6
// (Stirling numbers of the second kind S(6, k)).
__constant__ double kStirling6[7] = {0.0, 1.0, 31.0, 90.0, 65.0, 15.0, 1.0};

// Relabel rate classes in order of first appearance.
__device__ void rgs_normalize(int32_t *rc) {
    int32_t map[6] = {-1, -1, -1, -1, -1, -1}, next = 0;
    for (int i = 0; i < 6; ++i) {
        if (map[rc[i]] < 0) map[rc[i]] = next++;
        rc[i] = map[rc[i]];
    }
}

__device__ double ln_dirichlet(const double *alpha, const double *x, int n) {
    double s = 0.0, r = 0.0;
    for (int i = 0; i < n; ++i) {
        s += alpha[i];
        r += (alpha[i] - 1.0) * log(x[i]) - lgamma(alpha[i]);
    }
    return r + lgamma(s);
}

// Mixture members.  A member's prior density (in log) is the product of
// the parts its moves sample, as those moves' Hastings terms assume:
// weight and rate multiplier iid Exp(1); base frequencies equal (odds
// freqJumpPrior to estimated) or estimated with a flat Dirichlet prior
// (density 3! = 6); k rate classes with probability proportional to
// rateJumpPrior^-(k-1), a uniform partition among the S(6, k), class
// rates iid Exp(1); Gamma off (odds rateShapeInvJumpPrior to on) or 1/alpha
// ~ Exp(alpha_prior); +I off (odds invarJumpPrior to on) or wVar, wInvar ~
// Exp(1 - invarPrior), Exp(invarPrior).  A part no enabled move changes is
// the same in every member (slot 0's, copied) and adds nothing; a
// structural choice whose jump is disabled is slot 0's too.
__device__ inline bool mv_on(const Mc3Dev &d, int mv) { return (d.moves_on >> mv) & 1u; }

__device__ double mc3_member_lnprior(const Mc3Sub &q, const Mc3Dev &d) {
    double lp = -q.weight - q.rmult;
    if (mv_on(d, MV_FREQS) || mv_on(d, MV_FREQJ)) {
        if (mv_on(d, MV_FREQJ)) {
            const double f = d.freq_jump_prior;
            lp += q.freqs_est ? -log1p(f) : log(f) - log1p(f);
        }
        if (q.freqs_est) lp += 1.791759469228055;  // ln 3!
    }
    if (mv_on(d, MV_RATES) || mv_on(d, MV_RATE1) || mv_on(d, MV_RATEJ)) {
        double r[6];
        for (int i = 0; i < 6; ++i) r[q.rclass[i]] = q.rates[i];
        for (int c = 0; c < q.nrates; ++c) lp -= r[c];
        if (mv_on(d, MV_RATEJ)) {
            // P(k) = rjp^-(k-1) / sum_j rjp^-(j-1), then 1 / S(6, k).
            const double lr = log(d.rate_jump_prior);
            double z = 0.0;
            for (int j = 1; j <= 6; ++j) z += exp(-lr * (j - 1));
            lp += -lr * (q.nrates - 1) - log(z) - log(kStirling6[q.nrates]);
        }
    }
    if (d.ncat > 1 && (mv_on(d, MV_ALPHA) || mv_on(d, MV_GAMMAJ))) {
        if (mv_on(d, MV_GAMMAJ)) {
            const double g = d.gamma_jump_prior;
            lp += q.gamma_on ? -log1p(g) : log(g) - log1p(g);
        }
        if (q.gamma_on) lp += log(d.alpha_prior) - d.alpha_prior / q.alpha;
    }
    if (d.invar && (mv_on(d, MV_INVAR) || mv_on(d, MV_INVARJ))) {
        const bool on = q.winvar != 0.0;
        if (mv_on(d, MV_INVARJ)) {
            const double j = d.invar_jump_prior;
            lp += on ? -log1p(j) : log(j) - log1p(j);
        }
        if (on) {
            const double ip = d.invar_prior;
            lp += log(1.0 - ip) - (1.0 - ip) * q.wvar + log(ip) - ip * q.winvar;
        }
    }
    return lp;
}

// A new member drawn from that density (slot 0's member `ref` gives the
// fixed parts); returns its log density.
__device__ double mc3_draw_member(Mc3Sub &q, const Mc3Sub &ref, const Mc3Dev &d,
                                  Philox &rng) {
    auto expo = [&]() {
        const double x = -log(1.0 - philox_u01(rng));
        return x > 1e-300 ? x : 1e-300;
    };
    q = ref;
    q.weight = expo();
    q.rmult = expo();
    if (mv_on(d, MV_FREQS) || mv_on(d, MV_FREQJ)) {
        if (mv_on(d, MV_FREQJ))
            q.freqs_est = philox_u01(rng) < 1.0 / (1.0 + d.freq_jump_prior) ? 1 : 0;
        if (q.freqs_est) {
            double f[4], sum = 0.0;
            for (int i = 0; i < 4; ++i) sum += (f[i] = expo());
            for (int i = 0; i < 4; ++i) q.freqs[i] = f[i] / sum;
        } else {
            for (int i = 0; i < 4; ++i) q.freqs[i] = 0.25;
        }
    }
    if (mv_on(d, MV_RATES) || mv_on(d, MV_RATE1) || mv_on(d, MV_RATEJ)) {
        if (mv_on(d, MV_RATEJ)) {
            // k, then the r-th restricted growth string with k classes in
            // lexicographic order (203 strings in all).
            const double lr = log(d.rate_jump_prior);
            double z = 0.0, w[7];
            for (int j = 1; j <= 6; ++j) z += (w[j] = exp(-lr * (j - 1)));
            const double u = philox_u01(rng) * z;
            int k = 1;
            double acc = w[1];
            while (k < 6 && u >= acc) acc += w[++k];
            uint32_t r = philox_below(rng, (uint32_t)kStirling6[k]);
            int a[6] = {0, 0, 0, 0, 0, 0};
            for (int guard = 0; guard < 203; ++guard) {
                int mx = 0;
                for (int i = 0; i < 6; ++i) mx = a[i] > mx ? a[i] : mx;
                if (mx + 1 == k) {
                    if (r == 0) break;
                    --r;
                }
                // Next string: the rightmost a[i] below 1 + max(a[0..i-1])
                // goes up by one, the rest of the string to 0.
                int i = 5;
                for (; i >= 1; --i) {
                    int pm = 0;
                    for (int h = 0; h < i; ++h) pm = a[h] > pm ? a[h] : pm;
                    if (a[i] <= pm) break;
                }
                if (i < 1) break;
                ++a[i];
                for (int h = i + 1; h < 6; ++h) a[h] = 0;
            }
            for (int i = 0; i < 6; ++i) q.rclass[i] = a[i];
            q.nrates = k;
        }
        double cr[6];
        for (int c = 0; c < q.nrates; ++c) cr[c] = expo();
        for (int i = 0; i < 6; ++i) q.rates[i] = cr[q.rclass[i]];
    }
    if (d.ncat > 1 && (mv_on(d, MV_ALPHA) || mv_on(d, MV_GAMMAJ))) {
        if (mv_on(d, MV_GAMMAJ))
            q.gamma_on = philox_u01(rng) < 1.0 / (1.0 + d.gamma_jump_prior) ? 1 : 0;
        if (q.gamma_on) q.alpha = d.alpha_prior / expo();
    }
    if (d.invar && (mv_on(d, MV_INVAR) || mv_on(d, MV_INVARJ))) {
        bool on = q.winvar != 0.0;
        if (mv_on(d, MV_INVARJ)) on = philox_u01(rng) < 1.0 / (1.0 + d.invar_jump_prior);
        if (on) {
            q.wvar = expo() / (1.0 - d.invar_prior);
            q.winvar = expo() / d.invar_prior;
        } else {
            q.wvar = 1.0;
            q.winvar = 0.0;
        }
    }
    return mc3_member_lnprior(q, d);
}

// Member `from` (parameters and derived matrices) into slot `to`.
__device__ void mc3_move_member(Mc3Model &m, unsigned from, unsigned to) {
    m.q[to] = m.q[from];
    for (int i = 0; i < 4; ++i) m.pinorm[to * 4 + i] = m.pinorm[from * 4 + i];
    m.qnorm[to] = m.qnorm[from];
    for (int i = 0; i < 64; ++i) m.cube[to * 64 + i] = m.cube[from * 64 + i];
    for (int i = 0; i < 4; ++i) m.eig[to * 4 + i] = m.eig[from * 4 + i];
}

// Polytomies.  The chain's tree stays binary; an internal edge may be
// contracted (coll, length 0), and the multifurcating tree it stands for
// merges the edge's two ends.  The state is the multifurcating tree T'
// with a binary resolution R of each polytomy, and the target puts R
// uniform given T': the reference's prior on T' (polytomyJumpPrior per
// contracted edge, Exp(brlenPrior) lengths of the others) divided by
// NR(T'), the number of resolutions, prod over polytomies of (2d - 5)!!
// for degree d.  Every topology move adds ln NR(before) - ln NR(after) to
// its prior term.  A T' node merging c binary nodes has degree c + 2, so
// ln NR = sum over those sets of ln (2c - 1)!!.  uf and cnt are scratch
// ([nnodes] and [nnodes - ntaxa]).
__device__ double log_nresolutions(const int32_t *parent, const uint8_t *coll, int32_t *uf,
                                   int32_t *cnt, unsigned N, unsigned NN) {
    for (unsigned v = N; v < NN; ++v) {
        uf[v] = (int32_t)v;
        cnt[v - N] = 0;
    }
    auto find = [&](int v) {
        while (uf[v] != v) {
            uf[v] = uf[uf[v]];
            v = uf[v];
        }
        return v;
    };
    for (unsigned v = N; v < NN; ++v)
        if (coll[v] && parent[v] >= 0) {
            const int a = find((int)v), b = find(parent[v]);
            if (a != b) uf[a] = b;
        }
    for (unsigned v = N; v < NN; ++v) cnt[find((int)v) - (int)N]++;
    double s = 0.0;
    for (unsigned i = 0; i < NN - N; ++i)
        for (int k = 2; k <= cnt[i]; ++k) s += log(2.0 * k - 1.0);
    return s;
}

// One end of an eTBR move (Chain.pyx:517-597 for the X end, the same for
// Y) on a binary tree held as incidence lists: inc[v][0..2] are the edges
// at node v (-1: none) and ex[e] is the XOR of edge e's two end nodes, so
// the node across e from v is ex[e] ^ v.  From node n0 of edge eA: pick
// one of n0's other edges (eX), walk to its far node, and while that node
// is internal, extend with probability pext along a uniform edge other
// than the one just walked.  When the walk went past eX's far node n1,
// the rearrangement moves n0's sibling edge s to n1, eX to the
// second-to-last node r1 of the walk, and the last edge eR to n0, so n0
// (with eA) sits inside eR.  Lengths travel with their edges.
//
// ln q(back)/q(forth): the walk that undoes the move runs from n0 along eX
// back to n1 and ends across s, so it stops at s's far node as this walk
// stops at its last node, r0: each stop costs (1 - pext) at an internal
// node and nothing at a leaf.  (The reference conditions that term on the
// other end of eA, Chain.pyx:723-736; the ratio here is the one under
// which a chain on an empty alignment samples topologies uniformly, which
// tests check.)
struct EtbrEnd {
    int eX;      // first edge of the walk, -1 when n0 is a leaf
    double lnq;  // ln of the proposal ratio of this end's walk
};

__device__ inline int etbr_deg(const int32_t *inc, int v) {
    return (inc[v * 3] >= 0) + (inc[v * 3 + 1] >= 0) + (inc[v * 3 + 2] >= 0);
}

__device__ inline int etbr_pick(const int32_t *inc, int v, int ein, Philox &rng) {
    int cand[3], n = 0;
    for (int j = 0; j < 3; ++j) {
        const int e = inc[v * 3 + j];
        if (e >= 0 && e != ein) cand[n++] = e;
    }
    return cand[n > 1 ? philox_below(rng, (uint32_t)n) : 0];
}

__device__ inline void etbr_swap_edge(int32_t *inc, int v, int eold, int enew) {
    for (int j = 0; j < 3; ++j)
        if (inc[v * 3 + j] == eold) {
            inc[v * 3 + j] = enew;
            return;
        }
}

__device__ EtbrEnd etbr_end(int n0, int eA, int32_t *inc, int32_t *ex, Philox &rng,
                            double pext) {
    EtbrEnd r{-1, 0.0};
    if (etbr_deg(inc, n0) <= 1) return r;
    const int eX = etbr_pick(inc, n0, eA, rng);
    r.eX = eX;
    const int n1 = ex[eX] ^ n0;
    int e_last = eX, r1 = n0, r0 = n1;
    while (etbr_deg(inc, r0) > 1) {
        if (pext < philox_u01(rng)) break;
        const int e = etbr_pick(inc, r0, e_last, rng);
        r1 = r0;
        r0 = ex[e] ^ r0;
        e_last = e;
    }
    if (r0 == n1) return r;  // the walk did not leave eX: nothing moves
    int s = -1;
    for (int j = 0; j < 3; ++j) {
        const int e = inc[n0 * 3 + j];
        if (e >= 0 && e != eA && e != eX) s = e;
    }
    const int cs = ex[s] ^ n0;
    const int eR = e_last;
    // s: n0 -> n1; eX: n1 -> r1; eR: r1 -> n0 (in this order, each node
    // keeps three edges; r1 may be n1).
    etbr_swap_edge(inc, n1, eX, s);
    ex[s] ^= n0 ^ n1;
    etbr_swap_edge(inc, n0, s, eR);
    etbr_swap_edge(inc, r1, eR, eX);
    ex[eX] ^= n1 ^ r1;
    ex[eR] ^= r1 ^ n0;
    const double l1m = log1p(-pext);
    r.lnq = (etbr_deg(inc, cs) > 1 ? l1m : 0.0) - (etbr_deg(inc, r0) > 1 ? l1m : 0.0);
    return r;
}

// Shared memory of one chain's proposal: the tree (parent, child, len,
// cur), dirty flags, DFS stack, dirty list, the per-op prefix of
// children, and the stack slot of each op and of each op's children.
__host__ __device__ inline size_t mc3_propose_smem(unsigned NN, unsigned M) {
    return (size_t)NN * (8 + 4 + 12 + 4 + 1 + 1 + 1) + (size_t)M * 4 + (size_t)(M + 1) * 4 +
           (size_t)M * 4 + 64;
}

// One block per chain.  The chain's tree is staged in shared memory; one
// thread draws and applies the move and lists the dirty nodes there (the
// serial part: pointer chasing at shared-memory latency), then the block
// writes the op records and the tree back in parallel.
__global__ void mc3_propose_kernel(Mc3Dev d) {
    const unsigned c = blockIdx.x;
    if (c >= d.nchains) return;
    const uint64_t g = *d.gen;
    const unsigned N = d.ntaxa, NN = d.nnodes, M = d.M;
    extern __shared__ __align__(16) unsigned char psm[];
    double *len = reinterpret_cast<double *>(psm);
    int32_t *parent = reinterpret_cast<int32_t *>(len + NN);
    int32_t *child = parent + NN;
    int32_t *stack = child + (size_t)NN * 3;
    int32_t *dirty = stack + NN;
    uint32_t *kid0 = reinterpret_cast<uint32_t *>(dirty + M);   // [M + 1]
    uint8_t *cur = reinterpret_cast<uint8_t *>(kid0 + (M + 1));
    uint8_t *dflag = cur + NN;
    int8_t *op_slot = reinterpret_cast<int8_t *>(dflag + NN);   // [M]
    int8_t *kid_slot = op_slot + M;                             // [M][3]
    uint8_t *coll = reinterpret_cast<uint8_t *>(kid_slot + (size_t)M * 3);  // [NN]
    const unsigned tb = d.curtree[c];
    const size_t t_cur = (size_t)tb * d.nchains + c, t_alt = (size_t)(1 - tb) * d.nchains + c;
    int32_t *g_parent = d.parent + t_cur * NN;
    int32_t *g_child = d.child + t_cur * NN * 3;
    double *g_len = d.len + t_cur * NN;
    int32_t *a_child = d.child + t_alt * NN * 3;
    double *a_len = d.len + t_alt * NN;
    uint8_t *a_coll = d.coll + t_alt * NN;
    for (unsigned i = threadIdx.x; i < NN; i += blockDim.x) {
        len[i] = g_len[i];
        parent[i] = g_parent[i];
        cur[i] = d.cur[(size_t)c * NN + i];
        dflag[i] = 0;
        coll[i] = d.coll[t_cur * NN + i];
    }
    for (unsigned i = threadIdx.x; i < NN * 3; i += blockDim.x) child[i] = g_child[i];
    __syncthreads();
    Mc3Prop &pr = d.prop[c];
    {
        // The previous generation's accepted move: its dirty nodes' spare
        // CL buffers become current.
        const int prev_acc = pr.accepted, prev_nd = pr.ndirty;
        if (prev_acc)
            for (int i = threadIdx.x; i < prev_nd; i += blockDim.x)
                cur[d.dirty[(size_t)c * M + i]] ^= 1;
        // A model move edits the spare model slot, which starts as a copy
        // of the current one: copied here by the whole block (a struct
        // copy by the deciding thread alone took tens of microseconds).
        if (g > 0 && (d.moves_on & kModelMoves)) {
            static_assert(sizeof(Mc3Model) % 8 == 0, "model slots copy in 8-byte words");
            const unsigned long long *src =
                reinterpret_cast<const unsigned long long *>(&d.model[c * 2 + d.curmodel[c]]);
            unsigned long long *dst =
                reinterpret_cast<unsigned long long *>(&d.model[c * 2 + (1 - d.curmodel[c])]);
            for (unsigned i = threadIdx.x; i < sizeof(Mc3Model) / 8; i += blockDim.x)
                dst[i] = src[i];
        }
        __syncthreads();
    }
    __shared__ int s_nd, s_lowest, s_fl;
    __shared__ unsigned s_fin, s_fin_mi;
    __shared__ bool s_full, s_etbr;
    if (threadIdx.x == 0) {
        s_fin = 0;
        s_etbr = false;
        Philox rng;
        philox_init(rng, d.seed, c, g);
        if (c == 0) *d.counter = 0;
        char *res = d.results + (size_t)c * 32;
        // A walker tile that gave up on a bounded wait leaves the ticket
        // counted short; the error word stays set until the run reports it.
        *(uint32_t *)(res + 0) = 0;  // ticket
        *(uint32_t *)(res + 4) = 0;  // ninf

        const Mc3Model &m0 = d.model[c * 2 + d.curmodel[c]];
        Mc3Model &m1 = d.model[c * 2 + (1 - d.curmodel[c])];
        pr.model_changed = 0;
        pr.lnPrior = 0.0;
        pr.lnHast = 0.0;
        unsigned mi = 0;  // the mixture member a model move changes
        bool full = false;
        bool topo = false;  // a topology move under polytomy jumps
        double lnr0 = 0.0;  // ln NR of the current tree (topo)
        int lowest = -1;  // lowest dirty node of a path move
        if (g == 0) {
            pr.type = MV_INIT;
            full = true;
        } else {
            const double u = philox_u01(rng);
            int t = 0;
            while (t < kMoves - 1 && u >= d.wcdf[t]) ++t;
            if ((t == MV_NNI || t == MV_SPR) && N < 4) t = MV_BRLEN;
            // A model move acts on one uniform member of the mixture
            // (drawn only when there are several).
            const int nm = m0.nmodels;
            mi = nm > 1 ? philox_below(rng, (uint32_t)nm) : 0u;
            const Mc3Sub &q0 = m0.q[mi];
            // A move with nothing to change in this state is a branch
            // move instead, so each jump is drawn with the same
            // probability on both of its sides.
            if (t == MV_ALPHA && (d.ncat < 2 || !q0.gamma_on)) t = MV_BRLEN;
            if ((t == MV_INVAR && (!d.invar || q0.winvar == 0.0)) ||
                (t == MV_INVARJ && !d.invar))
                t = MV_BRLEN;
            if ((t == MV_RATES || t == MV_RATE1) && q0.nrates < 2) t = MV_BRLEN;
            if (t == MV_GAMMAJ && d.ncat < 2) t = MV_BRLEN;
            if (t == MV_FREQS && !q0.freqs_est) t = MV_BRLEN;
            if ((t == MV_WEIGHT || t == MV_RMULT) && nm < 2) t = MV_BRLEN;
            if (t == MV_MIXJ && d.mmax < 2) t = MV_BRLEN;
            if (t == MV_POLYJ && N < 4) t = MV_BRLEN;
            pr.type = t;
            topo = d.poly && (t == MV_NNI || t == MV_SPR || t == MV_ETBR || t == MV_POLYJ);
            if (topo) lnr0 = log_nresolutions(parent, coll, stack, dirty, N, NN);
            if (t == MV_BRLEN) {
                // Uniform edge = uniform non-root node (Chain.pyx:442-447)
                // that is not contracted.
                unsigned ncol = 0;
                if (d.poly)
                    for (unsigned v = N; v < NN; ++v) ncol += coll[v];
                unsigned k = philox_below(rng, NN - 1 - ncol);
                unsigned e = (k >= d.root) ? k + 1 : k;
                if (ncol) {
                    for (e = 0; e < NN; ++e) {
                        if (e == d.root || coll[e]) continue;
                        if (k-- == 0) break;
                    }
                }
                const double lnM = d.brlen_lambda * (philox_u01(rng) - 0.5);
                const double v0 = len[e], v1 = v0 * exp(lnM);
                len[e] = v1;
                pr.node = (int)e;
                pr.oldlen = v0;
                pr.lnPrior = -d.brlen_prior * (v1 - v0);
                pr.lnHast = lnM;
                lowest = parent[e];
            } else if (t == MV_NNI) {
                // Internal non-root node v, edge (v, p): swap a child a of v
                // with a sibling c of v (another child of p).
                unsigned k = philox_below(rng, M - 1);  // internal ids N..NN-1 minus root
                unsigned v = N + k;
                if (v >= d.root) ++v;
                const int p = parent[v];
                const int ai = (int)philox_below(rng, 2);
                const int a = child[v * 3 + ai];
                int sib[2], ns = 0;
                for (int j = 0; j < 3; ++j) {
                    const int x = child[p * 3 + j];
                    if (x >= 0 && x != (int)v) sib[ns++] = x;
                }
                const int cc = sib[ns > 1 ? philox_below(rng, ns) : 0];
                for (int j = 0; j < 3; ++j) {
                    if (child[v * 3 + j] == a) child[v * 3 + j] = cc;
                    if (child[p * 3 + j] == cc) child[p * 3 + j] = a;
                }
                parent[a] = p;
                parent[cc] = (int)v;
                pr.node = (int)v;
                pr.a = a;
                pr.c = cc;
                lowest = (int)v;
            } else if (t == MV_SPR) {
                // Subtree s: uniform over non-root nodes whose parent is not
                // the root (the root keeps its three children).
                const unsigned ns = NN - 1 - 3;
                unsigned k = philox_below(rng, ns);
                int s = -1;
                for (unsigned v = 0; v < NN && s < 0; ++v) {
                    if (v == d.root || parent[v] == (int)d.root) continue;
                    if (k-- == 0) s = (int)v;
                }
                const int p = parent[s], g = parent[p];
                int jb = -1, jg = -1;
                for (int j = 0; j < 3; ++j) {
                    const int x = child[p * 3 + j];
                    if (x >= 0 && x != s) jb = j;
                    if (child[g * 3 + j] == p) jg = j;
                }
                const int b = child[p * 3 + jb];
                // Mark the subtree of s (2 in the dirty flags, cleared below).
                unsigned nsub = 0;
                {
                    int sp = 0;
                    stack[sp++] = s;
                    while (sp > 0) {
                        const int v = stack[--sp];
                        dflag[v] = 2;
                        ++nsub;
                        for (int j = 0; j < 3; ++j) {
                            const int x = child[v * 3 + j];
                            if (x >= 0) stack[sp++] = x;
                        }
                    }
                }
                // Prune: b takes p's place under g, the two edges merge.
                pr.lb = len[b];
                pr.lp = len[p];
                child[g * 3 + jg] = b;
                parent[b] = g;
                len[b] = pr.lb + pr.lp;
                // Target edge (x, parent[x]) of the pruned tree, outside the
                // subtree: not the root, not p, not marked.
                const unsigned ne = NN - 2 - nsub;
                k = philox_below(rng, ne);
                int x = -1;
                for (unsigned v = 0; v < NN && x < 0; ++v) {
                    if (v == d.root || (int)v == p || dflag[v] == 2) continue;
                    if (k-- == 0) x = (int)v;
                }
                {
                    int sp = 0;
                    stack[sp++] = s;
                    while (sp > 0) {
                        const int v = stack[--sp];
                        dflag[v] = 0;
                        for (int j = 0; j < 3; ++j) {
                            const int y = child[v * 3 + j];
                            if (y >= 0) stack[sp++] = y;
                        }
                    }
                }
                const int xp = parent[x];
                int jx = -1;
                for (int j = 0; j < 3; ++j)
                    if (child[xp * 3 + j] == x) jx = j;
                const double lx = len[x];
                pr.lx = (x == b) ? pr.lb : lx;
                // Regraft p on (x, xp) at a uniform point.
                const double u = philox_u01(rng);
                child[xp * 3 + jx] = p;
                parent[p] = xp;
                child[p * 3 + jb] = x;
                parent[x] = p;
                len[p] = u * lx;
                len[x] = (1.0 - u) * lx;
                pr.s = s;
                pr.p = p;
                pr.g = g;
                pr.b = b;
                pr.x = x;
                pr.xp = xp;
                pr.jg = jg;
                pr.jb = jb;
                pr.jx = jx;
                pr.lnHast = (lx > 0.0) ? log(lx) - log(pr.lb + pr.lp) : 0.0;
                pr.lnPrior = (lx > 0.0) ? 0.0 : -INFINITY;
                // The edges whose lengths SPR merges and splits must be
                // real ones (it never changes contraction flags, so its
                // reverse meets the same edges).
                if (coll[p] || coll[b] || coll[x]) pr.lnPrior = -INFINITY;
                // Dirty: both paths to the root (p's new place, g's old child).
                for (int v = p; v >= 0; v = parent[v]) dflag[v] = 1;
                for (int v = g; v >= 0; v = parent[v]) dflag[v] = 1;
            } else if (t == MV_ETBR) {
                // Edges are named by the node below them in the current
                // rooting; len[] holds their lengths.  child[] becomes the
                // incidence lists and stack[] the end-node XORs.
                int32_t *inc = child, *ex = stack;
                for (unsigned v = 0; v < NN; ++v) {
                    if (v == d.root) continue;
                    int j = 0;
                    while (inc[v * 3 + j] >= 0) ++j;
                    inc[v * 3 + j] = (int)v;
                    ex[v] = (int)v ^ parent[v];
                }
                unsigned k = philox_below(rng, NN - 1);
                const int eA = (int)((k >= d.root) ? k + 1 : k);
                const int nX0 = eA, nY0 = ex[eA] ^ eA;
                const EtbrEnd X = etbr_end(nX0, eA, inc, ex, rng, d.etbr_pext);
                const EtbrEnd Y = etbr_end(nY0, eA, inc, ex, rng, d.etbr_pext);
                double lnH = X.lnq + Y.lnq, lnP = 0.0;
                const int em[3] = {eA, X.eX, Y.eX};
                for (int q = 0; q < 3; ++q) {
                    // A contracted edge keeps length 0 (no multiplier).
                    if (em[q] < 0 || coll[em[q]]) continue;
                    const double lnM = d.brlen_lambda * (philox_u01(rng) - 0.5);
                    const double v0 = len[em[q]], v1 = v0 * exp(lnM);
                    len[em[q]] = v1;
                    lnH += lnM;
                    lnP += -d.brlen_prior * (v1 - v0);
                }
                pr.lnPrior = lnP;
                pr.lnHast = lnH;
                // Root the result at the same node again, by an Euler
                // walk: parent[] gets the new parents, the spare buffer the
                // new child slots (-1 where the slot held the parent edge)
                // and lengths; dflag[v] is v's next incidence slot.
                parent[d.root] = -1;
                a_len[d.root] = len[d.root];
                a_coll[d.root] = 0;
                int v = (int)d.root;
                // The walk takes 3 NN slot steps and NN - 1 steps back up;
                // the bound only guards against a malformed tree.
                unsigned steps = 0;
                const unsigned max_steps = 4 * NN + 4;
                for (; steps < max_steps; ++steps) {
                    if (dflag[v] < 3) {
                        const int j = dflag[v]++;
                        const int e = inc[v * 3 + j];
                        const int u = e >= 0 ? (ex[e] ^ v) : -1;
                        if (u < 0 || u == parent[v]) {
                            a_child[v * 3 + j] = -1;
                            continue;
                        }
                        a_child[v * 3 + j] = u;
                        parent[u] = v;
                        a_len[u] = len[e];
                        a_coll[u] = coll[e];
                        v = u;
                    } else {
                        if (v == (int)d.root) break;
                        v = parent[v];
                    }
                }
                if (steps < max_steps) {
                    s_etbr = true;
                } else {
                    // Not reachable for a binary tree: report it, put the
                    // current tree back and reject the move.
                    atomicOr(d.status, 2u);
                    for (unsigned i = 0; i < NN; ++i) {
                        len[i] = g_len[i];
                        parent[i] = g_parent[i];
                        dflag[i] = 0;
                    }
                    for (unsigned i = 0; i < NN * 3; ++i) child[i] = g_child[i];
                    pr.lnPrior = -INFINITY;
                    lowest = (int)d.root;
                }
            } else if (t == MV_INVAR) {
                // Multiplier on wVar or wInvar (invarPropose,
                // Chain.pyx:379-436): Exp(1 - invarPrior) and
                // Exp(invarPrior) priors, Hastings ln m.
                const unsigned which = philox_below(rng, 2);
                const double lnM = d.invar_lambda * (philox_u01(rng) - 0.5);
                Mc3Sub &q1 = m1.q[mi];
                double &w = which == 0 ? q1.wvar : q1.winvar;
                const double w0 = w, w1 = w0 * exp(lnM);
                w = w1;
                pr.lnPrior = -(which == 0 ? 1.0 - d.invar_prior : d.invar_prior) * (w1 - w0);
                pr.lnHast = lnM;
                pr.model_changed = 1;
                s_fin = FIN_WEIGHTS;
                full = true;
            } else if (t == MV_INVARJ) {
                // +I off or on (invarJumpPropose, Chain.pyx:1449-1546).  Off
                // is wInvar = 0 with wVar = 1, as the reference's removal
                // leaves it; the +I component stays in the layout with
                // weight 0.  On, (wVar, wInvar) have the priors of the +I
                // weight move, Exp of rates 1 - invarPrior and invarPrior
                // (Chain.pyx:418-421), and adding draws them from those
                // priors, so the prior and proposal densities cancel in the
                // unheated chain; they are split between lnPrior and lnHast
                // as the reference splits its terms.  (The reference draws
                // added weights with means 1 - invarPrior and invarPrior,
                // which is not the density its weight move and prior use.)
                const double ip = d.invar_prior;
                Mc3Sub &q1 = m1.q[mi];
                auto lnw = [&](double wv, double wi) {
                    return log(1.0 - ip) - (1.0 - ip) * wv + log(ip) - ip * wi;
                };
                if (q0.winvar != 0.0) {
                    const double dens = lnw(q0.wvar, q0.winvar);
                    q1.wvar = 1.0;
                    q1.winvar = 0.0;
                    pr.lnPrior = log(d.invar_jump_prior) - dens;
                    pr.lnHast = dens;
                } else {
                    const double wv = -log(1.0 - philox_u01(rng)) / (1.0 - ip);
                    const double wi = -log(1.0 - philox_u01(rng)) / ip;
                    const double dens = lnw(wv, wi);
                    q1.wvar = wv;
                    q1.winvar = wi > 0.0 ? wi : 1e-300;
                    pr.lnPrior = -log(d.invar_jump_prior) + dens;
                    pr.lnHast = -dens;
                }
                pr.model_changed = 1;
                s_fin = FIN_WEIGHTS;
                full = true;
            } else if (t == MV_RATE1) {
                // One class rate times m = exp(lambda (u - 1/2)), Exp(1)
                // prior (ratePropose, Chain.pyx:267-319).
                const int r = (int)philox_below(rng, (uint32_t)q0.nrates);
                const double lnM = d.rate_lambda * (philox_u01(rng) - 0.5);
                double c0 = 0.0;
                for (int i = 0; i < 6; ++i)
                    if (q0.rclass[i] == r) c0 = q0.rates[i];
                const double c1 = c0 * exp(lnM);
                Mc3Sub &q1 = m1.q[mi];
                for (int i = 0; i < 6; ++i)
                    if (q0.rclass[i] == r) q1.rates[i] = c1;
                pr.lnPrior = -(c1 - c0);
                pr.lnHast = lnM;
                pr.model_changed = 1;
                s_fin = FIN_EIG;
                full = true;
            } else if (t == MV_RATEJ) {
                // Rate classes merged or split (rateJumpPropose,
                // rateMergePropose, rateSplitPropose, Chain.pyx:821-1075).
                // Prior (as the reference's randomLik draws it): k classes
                // with probability proportional to rateJumpPrior^-(k-1), a
                // uniform partition among the S(6, k), class rates iid
                // Exp(1).  Split: a uniform splittable class, a uniform
                // bipartition of its n0 members into non-empty parts A and
                // B, u uniform, rA = r0 n0 u / nA and rB = r0 n0 (1-u) / nB
                // (the member-weighted mean stays r0; Jacobian
                // n0^2 r0 / (nA nB)).  Merge: a uniform pair of classes to
                // their member-weighted mean.  Split or merge is chosen
                // with probability 1/2 where both exist.  The Hastings
                // terms are this scheme's own: the reference pre-assigns
                // two members to the parts and flips a coin for the rest,
                // which is not the uniform bipartition its proposal
                // ratio assumes.
                const int k = q0.nrates;
                int cnt[6] = {0, 0, 0, 0, 0, 0};
                double cr[6];
                for (int i = 0; i < 6; ++i) {
                    cnt[q0.rclass[i]]++;
                    cr[q0.rclass[i]] = q0.rates[i];
                }
                const bool merge =
                    k == 6 ? true : (k == 1 ? false : philox_below(rng, 2) == 0);
                const double lrjp = log(d.rate_jump_prior);
                Mc3Sub &q1 = m1.q[mi];
                if (!merge) {
                    int sp[6], ns = 0;
                    for (int r = 0; r < k; ++r)
                        if (cnt[r] > 1) sp[ns++] = r;
                    const int c = sp[philox_below(rng, (uint32_t)ns)];
                    const int n0 = cnt[c];
                    const uint32_t z = 1u + philox_below(rng, (1u << n0) - 2u);
                    const double u = philox_u01(rng), r0 = cr[c];
                    int nA = 0, j = 0;
                    for (int i = 0; i < 6; ++i)
                        if (q0.rclass[i] == c) nA += (z >> j++) & 1u;
                    const int nB = n0 - nA;
                    const double rA = r0 * n0 * u / nA, rB = r0 * n0 * (1.0 - u) / nB;
                    j = 0;
                    for (int i = 0; i < 6; ++i)
                        if (q0.rclass[i] == c) {
                            if ((z >> j++) & 1u) {
                                q1.rates[i] = rA;
                            } else {
                                q1.rclass[i] = k;
                                q1.rates[i] = rB;
                            }
                        }
                    rgs_normalize(q1.rclass);
                    q1.nrates = k + 1;
                    const double pS = k == 1 ? 1.0 : 0.5, pM = k + 1 == 6 ? 1.0 : 0.5;
                    pr.lnPrior = -lrjp + log(kStirling6[k]) - log(kStirling6[k + 1]) +
                                 (r0 - rA - rB);
                    pr.lnHast = (log(pM) - log(0.5 * (k + 1) * k)) -
                                (log(pS) - log((double)ns) - log((double)((1 << (n0 - 1)) - 1))) +
                                log((double)n0 * n0 * r0 / ((double)nA * nB));
                } else {
                    const int x = (int)philox_below(rng, (uint32_t)k);
                    int y = (int)philox_below(rng, (uint32_t)(k - 1));
                    if (y >= x) ++y;
                    const int a = x < y ? x : y, b = x < y ? y : x;
                    const int nA = cnt[a], nB = cnt[b], n0 = nA + nB;
                    const double rA = cr[a], rB = cr[b];
                    const double r0 = (nA * rA + nB * rB) / n0;
                    for (int i = 0; i < 6; ++i) {
                        int r = q0.rclass[i];
                        if (r == b) r = a;
                        else if (r > b) --r;
                        q1.rclass[i] = r;
                        if (r == a) q1.rates[i] = r0;
                    }
                    q1.nrates = k - 1;
                    int cnt1[6] = {0, 0, 0, 0, 0, 0}, ns1 = 0;
                    for (int i = 0; i < 6; ++i) cnt1[q1.rclass[i]]++;
                    for (int r = 0; r < k - 1; ++r) ns1 += cnt1[r] > 1;
                    const double pS = k - 1 == 1 ? 1.0 : 0.5, pM = k == 6 ? 1.0 : 0.5;
                    pr.lnPrior = lrjp + log(kStirling6[k]) - log(kStirling6[k - 1]) -
                                 (r0 - rA - rB);
                    pr.lnHast = (log(pS) - log((double)ns1) -
                                 log((double)((1 << (n0 - 1)) - 1))) -
                                (log(pM) - log(0.5 * k * (k - 1))) -
                                log((double)n0 * n0 * r0 / ((double)nA * nB));
                }
                pr.model_changed = 1;
                s_fin = FIN_EIG;
                full = true;
            } else if (t == MV_GAMMAJ) {
                // Gamma rates off or on (rateShapeInvJumpPropose,
                // Chain.pyx:1346-1450).  Adding draws 1/alpha from its
                // Exp(alpha_prior) prior; the prior and Jacobian terms are
                // split between lnPrior and lnHast as the reference does.
                const double sp = d.alpha_prior;
                Mc3Sub &q1 = m1.q[mi];
                if (q0.gamma_on) {
                    const double rsi0 = 1.0 / q0.alpha;
                    q1.gamma_on = 0;
                    pr.lnPrior = log(d.gamma_jump_prior) - log(sp) + sp * rsi0;
                    pr.lnHast = log(sp) - sp * rsi0;
                } else {
                    const double rsi1 = -log(1.0 - philox_u01(rng)) / sp;
                    q1.gamma_on = 1;
                    q1.alpha = 1.0 / rsi1;
                    pr.lnPrior = -log(d.gamma_jump_prior) + log(sp) - sp * rsi1;
                    pr.lnHast = -log(sp) + sp * rsi1;
                }
                pr.model_changed = 1;
                s_fin = FIN_GAMMA;
                full = true;
            } else if (t == MV_FREQJ) {
                // Equal or estimated base frequencies (freqJumpPropose,
                // Chain.pyx:1547-1631).  Estimated frequencies have a flat
                // Dirichlet prior (density 3! = 6 on the simplex), so
                // adding draws them from it: the density appears in
                // lnPrior and lnHast and cancels, as the reference's Exp(1)
                // terms do.
                const double ln6 = 1.791759469228055;
                Mc3Sub &q1 = m1.q[mi];
                if (q0.freqs_est) {
                    for (int i = 0; i < 4; ++i) q1.freqs[i] = 0.25;
                    q1.freqs_est = 0;
                    pr.lnPrior = log(d.freq_jump_prior) - ln6;
                    pr.lnHast = ln6;
                } else {
                    double f[4], s = 0.0;
                    for (int i = 0; i < 4; ++i) {
                        f[i] = -log(1.0 - philox_u01(rng));
                        if (f[i] < 1e-300) f[i] = 1e-300;
                        s += f[i];
                    }
                    for (int i = 0; i < 4; ++i) q1.freqs[i] = f[i] / s;
                    q1.freqs_est = 1;
                    pr.lnPrior = -log(d.freq_jump_prior) + ln6;
                    pr.lnHast = -ln6;
                }
                pr.model_changed = 1;
                s_fin = FIN_EIG;
                full = true;
            } else if (t == MV_FREQS) {
                // Base frequencies ~ Dirichlet(conc * pi).
                double f0[4], f1[4], a0[4], a1[4], s0 = 0.0, s1 = 0.0;
                for (int i = 0; i < 4; ++i) s0 += q0.freqs[i];
                for (int i = 0; i < 4; ++i) {
                    f0[i] = q0.freqs[i] / s0;
                    a0[i] = d.freq_conc * f0[i];
                    f1[i] = philox_gamma(rng, a0[i]);
                    if (f1[i] < 1e-300) f1[i] = 1e-300;
                    s1 += f1[i];
                }
                for (int i = 0; i < 4; ++i) {
                    f1[i] /= s1;
                    a1[i] = d.freq_conc * f1[i];
                }
                Mc3Sub &q1 = m1.q[mi];
                for (int i = 0; i < 4; ++i) q1.freqs[i] = f1[i];
                pr.lnHast = ln_dirichlet(a1, f0, 4) - ln_dirichlet(a0, f1, 4);
                pr.model_changed = 1;
                s_fin = FIN_EIG;
                full = true;
            } else if (t == MV_RATES) {
                // Class rates ~ Dirichlet(conc * r / sum r) over the k rate
                // classes, their sum kept (the rates' prior, iid Exp(1),
                // is flat Dirichlet in r / sum r and independent of the
                // sum).
                const int k = q0.nrates;
                double r0[6], r1[6], a0[6], a1[6], s0 = 0.0, s1 = 0.0;
                for (int i = 0; i < 6; ++i) r0[q0.rclass[i]] = q0.rates[i];
                for (int r = 0; r < k; ++r) s0 += r0[r];
                for (int r = 0; r < k; ++r) {
                    r0[r] /= s0;
                    a0[r] = d.rate_conc * r0[r];
                    r1[r] = philox_gamma(rng, a0[r]);
                    if (r1[r] < 1e-300) r1[r] = 1e-300;
                    s1 += r1[r];
                }
                for (int r = 0; r < k; ++r) {
                    r1[r] /= s1;
                    a1[r] = d.rate_conc * r1[r];
                }
                Mc3Sub &q1 = m1.q[mi];
                for (int i = 0; i < 6; ++i) q1.rates[i] = r1[q0.rclass[i]] * s0;
                pr.lnHast = ln_dirichlet(a1, r0, k) - ln_dirichlet(a0, r1, k);
                pr.model_changed = 1;
                s_fin = FIN_EIG;
                full = true;
            } else if (t == MV_POLYJ) {
                // An internal edge contracted or restored (polytomyJumpPropose,
                // polytomyMergePropose, polytomySplitPropose,
                // Chain.pyx:1076-1345).  Contract: a uniform internal edge
                // that is not contracted gets length 0.  Restore: a uniform
                // contracted edge gets a length drawn from its Exp(brlenPrior)
                // prior.  Each is the other's reverse; the choice between
                // them is 1/2 where both exist.  The prior ratio is the
                // reference's (polytomyJumpPrior and the edge's length
                // density); the resolution count NR follows below.
                unsigned nnc = 0, ncc = 0;
                for (unsigned w = N; w < NN; ++w) {
                    if (w == d.root) continue;
                    if (coll[w])
                        ++ncc;
                    else
                        ++nnc;
                }
                auto pcol = [](unsigned a, unsigned b) {
                    return a > 0 ? (b > 0 ? 0.5 : 1.0) : 0.0;
                };
                const bool col = nnc > 0 && (ncc == 0 || philox_below(rng, 2) == 0);
                unsigned k = philox_below(rng, col ? nnc : ncc);
                int v = -1;
                for (unsigned w = N; w < NN && v < 0; ++w) {
                    if (w == d.root || (coll[w] != 0) == col) continue;
                    if (k-- == 0) v = (int)w;
                }
                const double bp = d.brlen_prior, lpj = log(d.polytomy_jump_prior);
                pr.node = v;
                pr.oldlen = len[v];
                pr.a = coll[v];
                if (col) {
                    const double ld = log(bp) - bp * len[v];
                    coll[v] = 1;
                    len[v] = 0.0;
                    pr.lnPrior = lpj - ld;
                    pr.lnHast = log(pcol(ncc + 1, nnc - 1)) - log((double)(ncc + 1)) + ld -
                                (log(pcol(nnc, ncc)) - log((double)nnc));
                } else {
                    const double l = -log(1.0 - philox_u01(rng)) / bp;
                    const double ld = log(bp) - bp * l;
                    coll[v] = 0;
                    len[v] = l;
                    pr.lnPrior = -lpj + ld;
                    pr.lnHast = log(pcol(nnc + 1, ncc - 1)) - log((double)(nnc + 1)) - ld -
                                (log(pcol(ncc, nnc)) - log((double)ncc));
                }
                lowest = parent[v];
            } else if (t == MV_WEIGHT || t == MV_RMULT) {
                // A member's mixture weight or rate multiplier times
                // exp(lambda (u - 1/2)), Exp(1) prior, Hastings ln m
                // (weightPropose, rmultPropose, Chain.pyx:72-141, 200-266).
                const bool wt = t == MV_WEIGHT;
                const double lnM =
                    (wt ? d.weight_lambda : d.rmult_lambda) * (philox_u01(rng) - 0.5);
                double &x = wt ? m1.q[mi].weight : m1.q[mi].rmult;
                const double x0 = x, x1 = x0 * exp(lnM);
                x = x1;
                pr.lnPrior = -(x1 - x0);
                pr.lnHast = lnM;
                pr.model_changed = 1;
                s_fin = FIN_WEIGHTS;
                full = true;
            } else if (t == MV_MIXJ) {
                // A member added or removed (mixtureJumpPropose,
                // mixtureAddPropose, mixtureRemovePropose,
                // Chain.pyx:1633-1814).  Prior: k members with probability
                // proportional to (1 - mixJumpPrior)^(k-1), k <= mmax, each
                // drawn from mc3_member_lnprior's density.  Add draws the
                // new member from that density, appends it and swaps it
                // with a uniform slot j <= k; remove takes a uniform slot j,
                // moves the last member there and drops the last: the two
                // are each other's reverse with the same 1/(k+1) choice.
                // Add or remove is chosen with probability 1/2 where both
                // exist.  The member's density is in lnPrior and lnHast and
                // cancels in the unheated chain.
                const int k = m0.nmodels;
                auto p_add = [&](int n) { return n < (int)d.mmax ? (n > 1 ? 0.5 : 1.0) : 0.0; };
                auto p_rm = [&](int n) { return n > 1 ? (n < (int)d.mmax ? 0.5 : 1.0) : 0.0; };
                const bool add = k < (int)d.mmax && (k == 1 || philox_below(rng, 2) == 0);
                const double l1m = log1p(-d.mix_jump_prior);
                if (add) {
                    const unsigned j = philox_below(rng, (uint32_t)(k + 1));
                    Mc3Sub nq;
                    const double lnp = mc3_draw_member(nq, m0.q[0], d, rng);
                    if ((int)j < k) mc3_move_member(m1, j, (unsigned)k);
                    m1.q[j] = nq;
                    m1.nmodels = k + 1;
                    pr.lnPrior = l1m + lnp;
                    pr.lnHast = log(p_rm(k + 1)) - log(p_add(k)) - lnp;
                    s_fin = FIN_ALL;
                    s_fin_mi = j;
                } else {
                    const unsigned j = philox_below(rng, (uint32_t)k);
                    const double lnp = mc3_member_lnprior(m0.q[j], d);
                    if ((int)j + 1 < k) mc3_move_member(m1, (unsigned)(k - 1), j);
                    m1.nmodels = k - 1;
                    pr.lnPrior = -l1m - lnp;
                    pr.lnHast = log(p_add(k - 1)) - log(p_rm(k)) + lnp;
                    s_fin = FIN_WEIGHTS;
                    s_fin_mi = 0;
                }
                pr.model_changed = 1;
                full = true;
            } else {
                // Inverse Gamma shape multiplier (Chain.pyx:320-377).
                const double lnM = d.alpha_lambda * (philox_u01(rng) - 0.5);
                const double a0i = 1.0 / q0.alpha, a1i = a0i * exp(lnM);
                Mc3Sub &q1 = m1.q[mi];
                q1.alpha = 1.0 / a1i;
                pr.lnPrior = -d.alpha_prior * (a1i - a0i);
                pr.lnHast = lnM;
                pr.model_changed = 1;
                s_fin = FIN_GAMMA;
                full = true;
            }
        }
        if (topo && pr.lnPrior > -INFINITY) {
            // eTBR left the new tree's flags in the spare buffer.
            const double lnr1 = log_nresolutions(parent, pr.type == MV_ETBR ? a_coll : coll,
                                                 stack, dirty, N, NN);
            pr.lnPrior += lnr0 - lnr1;
        }
        if (pr.type != MV_MIXJ) s_fin_mi = mi;
        s_full = full;
        s_lowest = lowest;
    }
    __syncthreads();
    if (s_etbr) {
        // The re-rooted tree into shared memory.  A node whose children
        // are the same set as before keeps their old order; it is dirty if
        // the set or a child's edge length changed.
        for (unsigned v = threadIdx.x; v < NN; v += blockDim.x) {
            len[v] = a_len[v];
            coll[v] = a_coll[v];
            int nw[3] = {-1, -1, -1}, n = 0;
            for (int j = 0; j < 3; ++j) {
                const int x = a_child[v * 3 + j];
                if (x >= 0) nw[n++] = x;
            }
            int same = 1, nold = 0;
            for (int j = 0; j < 3; ++j) {
                const int x = g_child[v * 3 + j];
                if (x < 0) continue;
                ++nold;
                same &= (x == nw[0] || x == nw[1] || x == nw[2]);
            }
            same &= (nold == n);
            for (int j = 0; j < 3; ++j) child[v * 3 + j] = same ? g_child[v * 3 + j] : nw[j];
            dflag[v] = (v >= N && !same) ? 1 : 0;
        }
        __syncthreads();
        for (unsigned v = N + threadIdx.x; v < NN; v += blockDim.x) {
            if (dflag[v]) continue;
            for (int j = 0; j < 3; ++j) {
                const int u = child[v * 3 + j];
                if (u >= 0 && len[u] != g_len[u]) dflag[v] = 1;
            }
        }
        __syncthreads();
    }
    // The proposed model's derived quantities (a second warp) while thread
    // 0 lists the dirty nodes and assigns stack slots.
    if (threadIdx.x >= 32 && threadIdx.x < 64 && s_fin) {
        Mc3Model &m1 = d.model[c * 2 + (1 - d.curmodel[c])];
        const bool ok = mc3_model_finish_warp(m1, d.ncat, d.invar, d.mmax, s_fin, s_fin_mi);
        if (threadIdx.x == 32 && !ok) {
            // A model that cannot be decomposed is rejected outright.
            pr.lnPrior = -INFINITY;
            m1.ok = 0;
        }
    }
    if (threadIdx.x == 0) {
        const bool full = s_full;
        const int lowest = s_lowest;
        // Dirty internal nodes, children before parents.
        int nd = 0;
        if (s_etbr) {
            // Every ancestor of a changed node, and the root, is dirty too.
            dflag[d.root] = 1;
            for (unsigned v = N; v < NN; ++v) {
                if (dflag[v] != 1) continue;
                for (int u = parent[v]; u >= 0 && dflag[u] != 1; u = parent[u]) dflag[u] = 1;
            }
        }
        if (pr.type == MV_SPR || s_etbr) {
            // The nodes flagged above, in reversed pre-order of the new tree.
            int sp = 0;
            stack[sp++] = (int)d.root;
            while (sp > 0) {
                const int v = stack[--sp];
                if (dflag[v]) dirty[nd++] = v;
                for (int j = 0; j < 3; ++j) {
                    const int x = child[v * 3 + j];
                    if (x >= (int)N) stack[sp++] = x;
                }
            }
            for (int i = 0, j = nd - 1; i < j; ++i, --j) {
                const int t = dirty[i];
                dirty[i] = dirty[j];
                dirty[j] = t;
            }
        } else if (full && d.fl_nd[c] > 0) {
            // The kept full walk: the block copies it in below.
            nd = d.fl_nd[c];
        } else if (full) {
            // Iterative post-order from the root.
            int sp = 0, top = 0;
            stack[sp++] = (int)d.root;
            while (sp > 0) {
                const int v = stack[--sp];
                dirty[top++] = v;  // pre-order (parents first), reversed below
                for (int j = 0; j < 3; ++j) {
                    const int x = child[v * 3 + j];
                    if (x >= (int)N) stack[sp++] = x;
                }
            }
            // Reversed pre-order is a valid post-order (children first).
            for (int i = 0, j = top - 1; i < j; ++i, --j) {
                const int t = dirty[i];
                dirty[i] = dirty[j];
                dirty[j] = t;
            }
            nd = top;
        } else {
            for (int v = lowest; v >= 0; v = parent[v]) dirty[nd++] = v;
        }
        pr.ndirty = nd;
        s_fl = full ? (d.fl_nd[c] > 0 ? 1 : 2) : 0;  // 1: copy in, 2: keep
        if (s_fl == 1) {
            s_nd = nd;
        } else {
        for (int i = 0; i < nd; ++i) dflag[dirty[i]] = 1;

        // Children before each op (record layout).
        unsigned nk = 0;
        for (int o = 0; o < nd; ++o) {
            kid0[o] = nk;
            const int v = dirty[o];
            for (int j = 0; j < 3; ++j)
                if (child[v * 3 + j] >= 0) ++nk;
        }
        kid0[nd] = nk;
        // Shared-memory stack slots, as the host planner assigns them: a
        // result keeps a slot until its one consumer (a later op of this
        // walk) reads it; with no free slot the oldest holder loses its
        // slot and its consumer reads the HBM copy.  The DFS stack is free
        // now and maps a dirty node to its op.
        int32_t *op_of = stack;
        int owner[kMaxSlots];
        const int cap = (int)d.nslot_cap;
        for (int q = 0; q < cap; ++q) owner[q] = -1;
        for (int o = 0; o < nd; ++o) {
            const int v = dirty[o];
            int ci = 0;
            for (int j = 0; j < 3; ++j) {
                const int u = child[v * 3 + j];
                if (u < 0) continue;
                int ks = -1;
                if (u >= (int)N && dflag[u]) {
                    const int prod = op_of[u];
                    const int sl = op_slot[prod];
                    if (sl >= 0 && owner[sl] == prod) {
                        ks = sl;
                        owner[sl] = -1;
                    }
                }
                kid_slot[o * 3 + ci++] = (int8_t)ks;
            }
            op_of[v] = o;
            int sl = -1;
            if (o + 1 < nd && cap > 0) {
                for (int q = 0; q < cap && sl < 0; ++q)
                    if (owner[q] < 0) sl = q;
                if (sl < 0) {
                    sl = 0;
                    for (int q = 1; q < cap; ++q)
                        if (owner[q] < owner[sl]) sl = q;
                }
                owner[sl] = o;
            }
            op_slot[o] = (int8_t)sl;
        }
        s_nd = nd;
        }  // listed here
    }
    __syncthreads();
    const int nd = s_nd;
    if (s_fl != 0) {
        // A full walk of a topology seen before: order, children and slots
        // come from the chain's kept copy; a new one is kept for later.
        int32_t *fd = d.fl_dirty + (size_t)c * M;
        uint32_t *fk = d.fl_kid0 + (size_t)c * (M + 1);
        int8_t *fs = d.fl_slot + (size_t)c * 4 * M;
        if (s_fl == 1) {
            for (int i = threadIdx.x; i < nd; i += blockDim.x) {
                dirty[i] = fd[i];
                op_slot[i] = fs[i];
            }
            for (int i = threadIdx.x; i <= nd; i += blockDim.x) kid0[i] = fk[i];
            for (int i = threadIdx.x; i < 3 * nd; i += blockDim.x) kid_slot[i] = fs[M + i];
            for (unsigned v = N + threadIdx.x; v < NN; v += blockDim.x) dflag[v] = 1;
        } else {
            for (int i = threadIdx.x; i < nd; i += blockDim.x) {
                fd[i] = dirty[i];
                fs[i] = op_slot[i];
            }
            for (int i = threadIdx.x; i <= nd; i += blockDim.x) fk[i] = kid0[i];
            for (int i = threadIdx.x; i < 3 * nd; i += blockDim.x) fs[M + i] = kid_slot[i];
            __syncthreads();
            if (threadIdx.x == 0) d.fl_nd[c] = nd;
        }
        __syncthreads();
    }
    // Op records, one op per thread: parent -> its spare buffer; children
    // -> spare buffer if dirty (computed earlier in this walk), else
    // current.  A leaf child points at the leaf's mask array.
    const Mc3Model &mm = pr.model_changed ? d.model[c * 2 + (1 - d.curmodel[c])]
                                          : d.model[c * 2 + d.curmodel[c]];
    unsigned char *rec = d.rec + (size_t)c * M * d.rstride;
    const uint8_t **lrows = d.lrows + (size_t)c * M * 3;
    double *klen = d.kid_len + (size_t)c * d.maxkids;
    uint64_t *kdst = d.kid_dst + (size_t)c * d.maxkids;
    int32_t *ktab = d.kid_tab + (size_t)c * d.maxkids;
    for (int o = threadIdx.x; o < nd; o += blockDim.x) {
        const int v = dirty[o];
        const int mi = v - (int)N;
        unsigned char *r = rec + (size_t)o * d.rstride;
        RecHead hd;
        hd.data = d.cl_data[((size_t)c * M + mi) * 2 + (1 - cur[v])];
        hd.scaler = d.cl_sc[((size_t)c * M + mi) * 2 + (1 - cur[v])];
        const unsigned nch = kid0[o + 1] - kid0[o];
        hd.nchild = nch;
        hd.slot = op_slot[o];
        hd.flags = 0;
        hd.next_bytes = 0;
        int kcls[3] = {1, 1, 1};
        unsigned ci = 0, nkid = kid0[o], nl = 0;
        size_t area = sizeof(RecHead) + nch * sizeof(RecChild);
        const uint8_t **lr = lrows + (size_t)o * 3;
        for (int j = 0; j < 3; ++j) {
            const int u = child[v * 3 + j];
            if (u < 0) continue;
            RecChild ch;
            memset(&ch, 0, sizeof(ch));
            if (u < (int)N) {
                ch.data = d.leafmask[u];
                ch.idx = (uint32_t)u;  // staged row (leaf u is taxon u)
                lr[nl++] = d.leafmask[u];
                ch.src = SRC_LEAF;
                ch.tab = nkid;
                // FP64: table index; FP32: >= 0, the table goes in the record.
                ktab[nkid] = (int32_t)nkid;
            } else if (kid_slot[o * 3 + ci] >= 0) {
                ch.src = SRC_SLOT;
                ch.idx = (uint32_t)kid_slot[o * 3 + ci];
                ktab[nkid] = -1;
            } else {
                const int ui = u - (int)N;
                const int b = dflag[u] ? 1 - cur[u] : cur[u];
                ch.data = d.cl_data[((size_t)c * M + ui) * 2 + b];
                ch.scaler = d.cl_sc[((size_t)c * M + ui) * 2 + b];
                ch.src = SRC_GLOBAL;
                ktab[nkid] = -1;
            }
            ch.off = (uint32_t)area;
            memcpy(r + sizeof(RecHead) + ci * sizeof(RecChild), &ch, sizeof(ch));
            // Class for the op kind: dirty node o - 1 is F (its result is
            // still in the walker's registers).
            kcls[ci] = u < (int)N ? 0 : (o > 0 && u == dirty[o - 1] ? 2 : 1);
            klen[nkid] = len[u];
            kdst[nkid] = (size_t)o * d.rstride + area;
            area += child_area_bytes((int)d.prec, d.kact, u < (int)N);
            ++nkid;
            ++ci;
        }
        for (unsigned j = nl; j < 3; ++j) lr[j] = nullptr;
        if (d.prec == CXG_FP32 && nch == 2) hd.flags |= op_kind_of_classes(kcls[0], kcls[1]);
        memcpy(r, &hd, sizeof(hd));
    }
    // The tree (moved) and the dirty list back to HBM; an eTBR result goes
    // to the spare tree buffer, which the accept kernel makes current.
    {
        const size_t to = s_etbr ? t_alt : t_cur;
        int32_t *o_parent = d.parent + to * NN;
        int32_t *o_child = d.child + to * NN * 3;
        double *o_len = d.len + to * NN;
        uint8_t *o_coll = d.coll + to * NN;
        for (unsigned i = threadIdx.x; i < NN; i += blockDim.x) {
            o_len[i] = len[i];
            o_parent[i] = parent[i];
            o_coll[i] = coll[i];
        }
        for (unsigned i = threadIdx.x; i < NN * 3; i += blockDim.x) o_child[i] = child[i];
    }
    for (unsigned i = threadIdx.x; i < NN; i += blockDim.x) d.cur[(size_t)c * NN + i] = cur[i];
    for (int i = threadIdx.x; i < nd; i += blockDim.x)
        d.dirty[(size_t)c * M + i] = dirty[i];
    if (threadIdx.x == 0) {
        d.nkids[c] = kid0[nd];
        PlanArgs &job = d.jobs[c];
        job.nops = (uint32_t)nd;
        job.pn = mm.pn;
    }
}

// P matrices of every chain's child edges.
__global__ void mc3_pmat_kernel(Mc3Dev d) {
    // Four lanes per (chain, kid, comp), see pmat_one.
    const unsigned t = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const unsigned per = d.maxkids * d.kact;
    const unsigned c = t / per, r = t % per;
    if (c >= d.nchains || r >= d.nkids[c] * d.kact) return;
    const Mc3Prop &pr = d.prop[c];
    const Mc3Model &mm = d.model[c * 2 + (pr.model_changed ? 1 - d.curmodel[c]
                                                            : d.curmodel[c])];
    PmatArgs a;
    a.nchild = d.nkids[c];
    a.kact = d.kact;
    a.precision = (int)d.prec;
    a.edge_len = d.kid_len + (size_t)c * d.maxkids;
    a.cmult = mm.cmult;
    a.rmult = mm.rmult;
    a.model = mm.midx;
    a.cube = mm.cube;
    a.eig = mm.eig;
    a.dst = d.kid_dst + (size_t)c * d.maxkids;
    a.tab = d.kid_tab + (size_t)c * d.maxkids;
    a.wnorm = mm.wnorm;
    a.wnorm_dev = nullptr;
    a.rec = d.rec + (size_t)c * d.M * d.rstride;
    a.ltab = d.ltab + (size_t)c * d.maxkids * 16 * d.kact * 4;
    pmat_one(a, r, threadIdx.x & 3u);
}

// One block; thread c decides chain c, then thread 0 tries the heat swap.
__global__ void mc3_accept_kernel(Mc3Dev d) {
    if (blockIdx.x != 0) return;
    const uint64_t g = *d.gen;
    const unsigned N = d.ntaxa, NN = d.nnodes;
    for (unsigned c = threadIdx.x; c < d.nchains; c += blockDim.x) {
        Mc3Prop &pr = d.prop[c];
        const char *res = d.results + (size_t)c * 32;
        const uint32_t ninf = *(const uint32_t *)(res + 4);
        const double lnL1 = ninf ? -INFINITY
                                 : ((const double *)(res + 16))[0] +
                                       ((const double *)(res + 16))[1];
        bool accept;
        if (pr.type == MV_INIT) {
            accept = true;
        } else {
            Philox rng;
            philox_init(rng, d.seed, 0x40000000u + c, g);
            const double u = philox_u01(rng);
            // p = [(likelihood ratio)(prior ratio)]^heat * (Hastings ratio)
            const double p =
                exp(((lnL1 - d.lnL[c]) + pr.lnPrior) * d.heat[c] + pr.lnHast);
            accept = (p >= u) && (p > 0.0) && isfinite(lnL1);
        }
        // The dirty nodes' CL buffers flip in the next proposal kernel.
        pr.accepted = accept ? 1 : 0;
        if (accept) {
            d.lnL[c] = lnL1;
            if (pr.type == MV_NNI || pr.type == MV_SPR || pr.type == MV_ETBR) d.fl_nd[c] = 0;
            if (pr.model_changed) d.curmodel[c] ^= 1;
            if (pr.type == MV_ETBR) d.curtree[c] ^= 1;
            if (pr.type < kMoves) d.acc[c * kMoves + pr.type]++;
        } else {
            // A rejected eTBR move left the current tree buffer as it was.
            const size_t tc = (size_t)d.curtree[c] * d.nchains + c;
            int32_t *parent = d.parent + tc * NN;
            int32_t *child = d.child + tc * NN * 3;
            if (pr.type == MV_BRLEN) {
                d.len[tc * NN + pr.node] = pr.oldlen;
            } else if (pr.type == MV_POLYJ) {
                d.len[tc * NN + pr.node] = pr.oldlen;
                d.coll[tc * NN + pr.node] = (uint8_t)pr.a;
            } else if (pr.type == MV_SPR) {
                // Take p out of (x, xp), put it back between g and b.
                const int p = pr.p, x = pr.x, b = pr.b, g = pr.g, xp = pr.xp;
                double *len = d.len + tc * NN;
                child[xp * 3 + pr.jx] = x;
                parent[x] = xp;
                child[p * 3 + pr.jb] = b;
                parent[b] = p;
                child[g * 3 + pr.jg] = p;
                parent[p] = g;
                len[b] = pr.lb;
                len[p] = pr.lp;
                if (x != b) len[x] = pr.lx;
            } else if (pr.type == MV_NNI) {
                const int v = pr.node, a = pr.a, cc = pr.c;
                const int p = parent[a];
                for (int j = 0; j < 3; ++j) {
                    if (child[v * 3 + j] == cc) child[v * 3 + j] = a;
                    if (child[p * 3 + j] == a) child[p * 3 + j] = cc;
                }
                parent[a] = v;
                parent[cc] = p;
            }
            if (pr.type < kMoves) d.rej[c * kMoves + pr.type]++;
        }
        (void)N;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    // Heat swap between a random pair (Chain.pyx:1874-1911).
    if (d.nchains > 1 && g > 0 && g % d.swap_stride == 0) {
        Philox rng;
        philox_init(rng, d.seed, 0x7fffffffu, g);
        const unsigned a = philox_below(rng, d.nchains);
        unsigned b = philox_below(rng, d.nchains - 1);
        if (b >= a) ++b;
        const double u = philox_u01(rng);
        const double p = exp((d.lnL[b] - d.lnL[a]) * d.heat[a] +
                             (d.lnL[a] - d.lnL[b]) * d.heat[b]);
        if (p >= u) {
            const double t = d.heat[a];
            d.heat[a] = d.heat[b];
            d.heat[b] = t;
            d.nswap[a]++;
            d.nswap[b]++;
        }
    }
    if (g < d.trace_cap) {
        double cold = d.lnL[0];
        for (unsigned c = 0; c < d.nchains; ++c)
            if (d.heat[c] == 1.0) cold = d.lnL[c];
        d.trace[g] = cold;
    }
    *d.gen = g + 1;
}

}  // namespace cxg

using namespace cxg;

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct cxgMc3 {
    // Calls on one handle are serialised; separate handles (their own
    // streams, graphs and buffers) run concurrently.
    std::mutex mu;
    Mc3Dev d;
    cxgMc3Config cfg;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    BatchArgs ba;
    unsigned grid = 0, pmat_grid = 0;
    size_t propose_smem = 0;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    unsigned graph_gens = 0;
    double last_walk_ms = 0.0;
};

// The proposal kernel's dynamic shared-memory limit is one setting for
// every handle: it only grows, under one lock, so a smaller handle made
// later (or on another thread) never lowers it below what a larger one
// launches with.
static cudaError_t raise_propose_smem(size_t n) {
    static std::mutex mu;
    static size_t cur = 0;
    std::lock_guard<std::mutex> g(mu);
    if (n <= cur) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(
        mc3_propose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)n);
    if (e == cudaSuccess) cur = n;
    return e;
}

static int mc3_alloc(cxgMc3 *h, void **p, size_t n) {
    cudaError_t e = dev_malloc((void **)p, n ? n : 16);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(mc3)");
    h->allocs.push_back(*p);
    e = cudaMemset(*p, 0, n ? n : 16);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(mc3)");
    return 0;
}

template <typename T>
static int mc3_upload(cxgMc3 *h, T **dst, const T *src, size_t count) {
    int rc = mc3_alloc(h, (void **)dst, count * sizeof(T));
    if (rc) return rc;
    if (src) {
        cudaError_t e = cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(mc3)");
    }
    return 0;
}

static void mc3_free(cxgMc3 *h) {
    if (h->exec) cudaGraphExecDestroy(h->exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (void *p : h->allocs) dev_free(p);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

static int mc3_enqueue_gen(cxgMc3 *h) {
    const Mc3Dev &d = h->d;
    mc3_propose_kernel<<<d.nchains, 128, h->propose_smem, h->stream>>>(d);
    CXG_CHECK_LAUNCH("mc3_propose_kernel");
    mc3_pmat_kernel<<<h->pmat_grid, 128, 0, h->stream>>>(d);
    CXG_CHECK_LAUNCH("mc3_pmat_kernel");
    cudaError_t e = launch_batch((int)d.prec, h->ba, h->grid, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "walk_batch_kernel");
    mc3_accept_kernel<<<1, d.nchains < 1024 ? ((d.nchains + 31) / 32) * 32 : 1024, 0,
                        h->stream>>>(d);
    CXG_CHECK_LAUNCH("mc3_accept_kernel");
    return 0;
}

extern "C" int cxgMc3Create(const cxgMc3Config *cfg, cxgMc3 **out) {
    if (cfg == nullptr || out == nullptr) return fail(CXG_EINVAL, "cxgMc3Create: NULL");
    const unsigned N = cfg->ntaxa;
    if (N < 3 || N > 3000) return fail(CXG_EINVAL, "cxgMc3Create: 3..3000 taxa");
    if (!(cfg->pinv >= 0.0 && cfg->pinv < 1.0))
        return fail(CXG_EINVAL, "cxgMc3Create: pinv must be in [0, 1)");
    const unsigned invar = cfg->pinv > 0.0 ? 1u : 0u;
    const unsigned mmax = cfg->max_models ? cfg->max_models : 1u;
    if (mmax > (unsigned)kMaxModels)
        return fail(CXG_EINVAL, "cxgMc3Create: max_models must be 1..4");
    if (cfg->ncat < 1 || mmax * (cfg->ncat + invar) > kMaxComps)
        return fail(CXG_EINVAL,
                    "cxgMc3Create: 1..8 components (max_models x (rate categories, +I))");
    if (cfg->nchains < 1 || cfg->nchains > 1024)
        return fail(CXG_EINVAL, "cxgMc3Create: 1..1024 chains");
    if (cfg->precision != CXG_FP32 && cfg->precision != CXG_FP64)
        return fail(CXG_EINVAL, "unknown precision");
    if (cfg->npat == 0) return fail(CXG_EINVAL, "cxgMc3Create: no patterns");
    const unsigned NN = 2 * N - 2, M = N - 2;
    if (cfg->root < N || cfg->root >= NN)
        return fail(CXG_EINVAL, "cxgMc3Create: root must be an internal node");
    // Children from the parent array; check a binary rooted tree.
    std::vector<int32_t> child(NN * 3, -1);
    std::vector<int> nch(NN, 0);
    for (unsigned v = 0; v < NN; ++v) {
        const int p = cfg->parent[v];
        if (v == cfg->root) {
            if (p != -1) return fail(CXG_EINVAL, "root has a parent");
            continue;
        }
        if (p < (int)N || p >= (int)NN)
            return fail(CXG_EINVAL, "parent of a node must be an internal node");
        if (nch[p] >= 3) return fail(CXG_EINVAL, "node with more than 3 children");
        child[p * 3 + nch[p]++] = (int)v;
    }
    for (unsigned v = N; v < NN; ++v)
        if (nch[v] != (v == cfg->root ? 3 : 2))
            return fail(CXG_EINVAL, "tree is not binary (root degree 3)");
    cxgMc3 *h = new cxgMc3();
    h->cfg = *cfg;
    Mc3Dev &d = h->d;
    memset(&d, 0, sizeof(d));
    const unsigned C = cfg->nchains, K = mmax * (cfg->ncat + invar);
    d.ncat = cfg->ncat;
    d.invar = invar;
    d.kper = cfg->ncat + invar;
    d.mmax = mmax;
    d.nchains = C;
    d.ntaxa = N;
    d.nnodes = NN;
    d.root = cfg->root;
    d.kact = K;
    d.npat = cfg->npat;
    d.ppad = pad_patterns(cfg->npat);
    d.prec = (uint32_t)cfg->precision;
    d.M = M;
    d.maxkids = NN;  // children over all internal nodes: NN - 1
    const size_t elt = cfg->precision == CXG_FP32 ? 4 : 8;
    d.rstride = (uint32_t)((sizeof(RecHead) +
                            3 * (sizeof(RecChild) +
                                 std::max(child_area_bytes(cfg->precision, K, true),
                                          child_area_bytes(cfg->precision, K, false))) +
                            15) &
                           ~(size_t)15);
    unsigned tile = 0, tpp_q = 1;
    size_t budget = 0;
    unsigned ppt_q = 1;
    cxgTuneGet(&tile, &tpp_q, &ppt_q, &budget);
    const unsigned tpp = tuned_tpp(cfg->precision, K, tile);
    const unsigned ppt = tuned_ppt(cfg->precision, K, tile, tpp);
    d.ntiles = d.ppad / tile;
    {
        // Leaves staged per tile when they fit, else streamed with the op
        // records; stack slots within the tuned shared-memory budget.
        d.staged = (size_t)N * tile <= kLeafStageBytes;
        const unsigned lm = d.staged ? 0 : 3, nl = d.staged ? N : 0;
        const size_t base_b =
            plan_smem_bytes(cfg->precision, K, tile, 0, kRing, d.rstride, lm, nl);
        const size_t slot_b =
            plan_smem_bytes(cfg->precision, K, tile, 1, kRing, d.rstride, lm, nl) - base_b;
        size_t cap = budget > base_b ? (budget - base_b) / slot_b : 0;
        d.nslot_cap = (uint32_t)(cap > kMaxSlots ? kMaxSlots : cap);
    }
    d.seed = cfg->seed;
    d.swap_stride = cfg->swap_stride ? cfg->swap_stride : 1;
    // Without a +I component the +I weight move has nothing to change
    // (the reference disables PropInvar then, Mc3/__init__.pyx:934-937).
    double mw[kMoves], wsum = 0.0;
    for (int i = 0; i < kMoves; ++i) mw[i] = cfg->move_weight[i];
    if (!invar) mw[MV_INVAR] = mw[MV_INVARJ] = 0.0;
    for (int i = 0; i < kMoves; ++i) wsum += mw[i];
    if (!(wsum > 0.0)) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: all move weights are zero");
    }
    double acc = 0.0;
    for (int i = 0; i < kMoves; ++i) {
        acc += mw[i] / wsum;
        d.wcdf[i] = (i == kMoves - 1) ? 2.0 : acc;
        if (mw[i] > 0.0) d.moves_on |= 1u << i;
    }
    d.brlen_lambda = cfg->brlen_lambda;
    d.brlen_prior = cfg->brlen_prior;
    d.rate_conc = cfg->rate_conc;
    d.freq_conc = cfg->freq_conc > 0.0 ? cfg->freq_conc : 300.0;
    if (!(cfg->etbr_pext >= 0.0 && cfg->etbr_pext <= 1.0)) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: etbr_pext must be in [0, 1]");
    }
    d.etbr_pext = cfg->etbr_pext;
    d.alpha_lambda = cfg->alpha_lambda;
    d.alpha_prior = cfg->alpha_prior;
    d.invar_lambda = cfg->invar_lambda;
    d.invar_prior = cfg->invar_prior;
    d.gamma_jump_prior = cfg->gamma_jump_prior;
    d.freq_jump_prior = cfg->freq_jump_prior;
    d.invar_jump_prior = cfg->invar_jump_prior;
    d.rate_jump_prior = cfg->rate_jump_prior;
    d.rate_lambda = cfg->rate_lambda;
    d.mix_jump_prior = cfg->mixture_jump_prior;
    d.polytomy_jump_prior = cfg->polytomy_jump_prior;
    d.poly = mw[MV_POLYJ] > 0.0 ? 1u : 0u;
    if (d.poly && !(cfg->polytomy_jump_prior > 0.0)) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: polytomy_jump_prior must be positive");
    }
    d.weight_lambda = cfg->weight_lambda;
    d.rmult_lambda = cfg->rmult_lambda;
    if (mw[MV_MIXJ] > 0.0 && mmax > 1 &&
        !(cfg->mixture_jump_prior >= 0.0 && cfg->mixture_jump_prior < 1.0)) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: mixture_jump_prior must be in [0, 1)");
    }
    // Rate classes: a restricted growth string, equal rates within a class.
    int nrates = 0;
    for (int i = 0; i < 6; ++i) {
        const int r = cfg->rclass[i];
        if (r < 0 || r > nrates) {
            mc3_free(h);
            return fail(CXG_EINVAL, "cxgMc3Create: rclass is not a restricted growth string");
        }
        if (r == nrates) ++nrates;
        for (int j = 0; j < i; ++j)
            if (cfg->rclass[j] == r && cfg->rates[j] != cfg->rates[i]) {
                mc3_free(h);
                return fail(CXG_EINVAL,
                            "cxgMc3Create: rates of one rate class differ");
            }
    }
    if (mw[MV_RATEJ] > 0.0 && !(cfg->rate_jump_prior > 0.0)) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: rate_jump_prior must be positive");
    }
    if ((mw[MV_GAMMAJ] > 0.0 && !(cfg->gamma_jump_prior > 0.0)) ||
        (mw[MV_FREQJ] > 0.0 && !(cfg->freq_jump_prior > 0.0)) ||
        (mw[MV_INVARJ] > 0.0 && !(cfg->invar_jump_prior > 0.0))) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: jump priors must be positive");
    }
    if (invar && !(cfg->invar_prior > 0.0 && cfg->invar_prior < 1.0)) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: invar_prior must be in (0, 1)");
    }
    d.trace_cap = cfg->trace_cap;
    int rc = 0;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        mc3_free(h);
        return cuda_fail(e, "cudaStreamCreate(mc3)");
    }
    // Topology, lengths (both tree buffers of every chain), CL buffers.
    std::vector<int32_t> par_all((size_t)2 * C * NN), ch_all((size_t)2 * C * NN * 3);
    std::vector<double> len_all((size_t)2 * C * NN);
    for (unsigned c = 0; c < 2 * C; ++c) {
        memcpy(&par_all[(size_t)c * NN], cfg->parent, NN * 4);
        memcpy(&ch_all[(size_t)c * NN * 3], child.data(), NN * 3 * 4);
        memcpy(&len_all[(size_t)c * NN], cfg->len, NN * 8);
    }
    std::vector<double> heat(C), lnl(C, 0.0);
    for (unsigned c = 0; c < C; ++c) heat[c] = 1.0 / (1.0 + c * cfg->heat_delta);
    std::vector<Mc3Model> models((size_t)C * 2);
    for (auto &m : models) {
        memset(&m, 0, sizeof(m));
        m.nmodels = 1;
        Mc3Sub &q = m.q[0];
        for (int i = 0; i < 6; ++i) q.rates[i] = cfg->rates[i];
        for (int i = 0; i < 6; ++i) q.rclass[i] = cfg->rclass[i];
        q.nrates = nrates;
        for (int i = 0; i < 4; ++i) q.freqs[i] = cfg->freqs[i];
        q.alpha = cfg->alpha;
        q.wvar = invar ? 1.0 - cfg->pinv : 1.0;
        q.winvar = invar ? cfg->pinv : 0.0;
        q.gamma_on = cfg->ncat > 1 ? 1 : 0;
        // Equal frequencies start in the equal state (Chain.freqsEqual).
        q.freqs_est = !(cfg->freqs[0] == cfg->freqs[1] && cfg->freqs[1] == cfg->freqs[2] &&
                        cfg->freqs[2] == cfg->freqs[3]);
        q.weight = 1.0;
        q.rmult = 1.0;
    }
    // Leaf masks (0 = any state, as Lik.pyx:1469-1470), pattern weights.
    std::vector<uint8_t> masks((size_t)N * d.ppad, 15);
    for (unsigned t = 0; t < N; ++t)
        for (unsigned p = 0; p < cfg->npat; ++p) {
            const uint8_t v = cfg->masks[(size_t)t * cfg->npat + p] & 15;
            masks[(size_t)t * d.ppad + p] = v ? v : 15;
        }
    uint8_t *dmask = nullptr;
    uint32_t *dfreq = nullptr;
    const uint8_t **leafptr_host = new const uint8_t *[N];
    std::vector<void *> cl((size_t)C * M * 2), sc((size_t)C * M * 2);
    const size_t cl_bytes = (size_t)K * 4 * d.ppad * elt, sc_bytes = (size_t)d.ppad * 8;
    if ((rc = mc3_upload(h, &d.parent, par_all.data(), par_all.size())) ||
        (rc = mc3_upload(h, &d.child, ch_all.data(), ch_all.size())) ||
        (rc = mc3_upload(h, &d.len, len_all.data(), len_all.size())) ||
        (rc = mc3_upload<uint8_t>(h, &d.coll, nullptr, (size_t)2 * C * NN)) ||
        (rc = mc3_upload<uint8_t>(h, &d.curtree, nullptr, C)) ||
        (rc = mc3_upload<uint8_t>(h, &d.cur, nullptr, (size_t)C * NN)) ||
        (rc = mc3_upload<int32_t>(h, &d.dirty, nullptr, (size_t)C * M)) ||
        (rc = mc3_upload<int32_t>(h, &d.fl_nd, nullptr, C)) ||
        (rc = mc3_upload<int32_t>(h, &d.fl_dirty, nullptr, (size_t)C * M)) ||
        (rc = mc3_upload<uint32_t>(h, &d.fl_kid0, nullptr, (size_t)C * (M + 1))) ||
        (rc = mc3_upload<int8_t>(h, &d.fl_slot, nullptr, (size_t)C * 4 * M)) ||
        (rc = mc3_upload<int32_t>(h, &d.stack, nullptr, (size_t)C * NN)) ||
        (rc = mc3_upload(h, &d.model, models.data(), models.size())) ||
        (rc = mc3_upload<uint8_t>(h, &d.curmodel, nullptr, C)) ||
        (rc = mc3_upload(h, &d.lnL, lnl.data(), C)) ||
        (rc = mc3_upload(h, &d.heat, heat.data(), C)) ||
        (rc = mc3_upload<uint64_t>(h, &d.gen, nullptr, 1)) ||
        (rc = mc3_upload<Mc3Prop>(h, &d.prop, nullptr, C)) ||
        (rc = mc3_upload<PlanArgs>(h, &d.jobs, nullptr, C)) ||
        (rc = mc3_upload<unsigned char>(h, &d.rec, nullptr, (size_t)C * M * d.rstride)) ||
        (rc = mc3_upload<const uint8_t *>(h, (const uint8_t ***)&d.lrows, nullptr,
                                          (size_t)C * M * 3)) ||
        (rc = mc3_upload<double>(h, &d.kid_len, nullptr, (size_t)C * d.maxkids)) ||
        (rc = mc3_upload<uint64_t>(h, &d.kid_dst, nullptr, (size_t)C * d.maxkids)) ||
        (rc = mc3_upload<int32_t>(h, &d.kid_tab, nullptr, (size_t)C * d.maxkids)) ||
        (rc = mc3_upload<uint32_t>(h, &d.nkids, nullptr, C)) ||
        (rc = mc3_upload<double>(h, &d.ltab, nullptr,
                                 cfg->precision == CXG_FP64
                                     ? (size_t)C * d.maxkids * 16 * K * 4
                                     : 2)) ||
        (rc = mc3_upload<char>(h, &d.results, nullptr, (size_t)C * 32 + 16)) ||
        (rc = mc3_upload<uint32_t>(h, &d.acc, nullptr, (size_t)C * kMoves)) ||
        (rc = mc3_upload<uint32_t>(h, &d.rej, nullptr, (size_t)C * kMoves)) ||
        (rc = mc3_upload<uint32_t>(h, &d.nswap, nullptr, C)) ||
        (rc = mc3_upload<double>(h, &d.trace, nullptr, cfg->trace_cap ? cfg->trace_cap : 1)) ||
        (rc = mc3_upload<uint32_t>(h, &d.status, nullptr, 1)) ||
        (rc = mc3_upload(h, &dmask, masks.data(), masks.size())) ||
        (rc = mc3_upload(h, &dfreq, cfg->freqs_pattern, cfg->npat))) {
        delete[] leafptr_host;
        mc3_free(h);
        return rc;
    }
    for (unsigned t = 0; t < N; ++t) leafptr_host[t] = dmask + (size_t)t * d.ppad;
    rc = mc3_upload(h, (const uint8_t ***)&d.leafmask, leafptr_host, N);
    delete[] leafptr_host;
    if (rc) {
        mc3_free(h);
        return rc;
    }
    d.counter = (unsigned *)(d.results + (size_t)C * 32);
    {
        void *slab_cl = nullptr, *slab_sc = nullptr;
        if ((rc = mc3_alloc(h, &slab_cl, cl.size() * cl_bytes)) ||
            (rc = mc3_alloc(h, &slab_sc, sc.size() * sc_bytes))) {
            mc3_free(h);
            return rc;
        }
        for (size_t i = 0; i < cl.size(); ++i) {
            cl[i] = static_cast<char *>(slab_cl) + i * cl_bytes;
            sc[i] = static_cast<char *>(slab_sc) + i * sc_bytes;
        }
    }
    if ((rc = mc3_upload(h, &d.cl_data, cl.data(), cl.size())) ||
        (rc = mc3_upload(h, &d.cl_sc, sc.data(), sc.size()))) {
        mc3_free(h);
        return rc;
    }
    // Walk jobs: one per chain.
    double *partial = nullptr;
    if ((rc = mc3_upload<double>(h, &partial, nullptr, (size_t)C * d.ntiles * 2))) {
        mc3_free(h);
        return rc;
    }
    std::vector<PlanArgs> jobs(C);
    std::vector<WalkItem> items;
    for (unsigned c = 0; c < C; ++c) {
        PlanArgs a;
        memset(&a, 0, sizeof(a));
        a.rec = d.rec + (size_t)c * M * d.rstride;
        a.lrows = d.lrows + (size_t)c * M * 3;
        a.lmax = d.staged ? 0 : 3;
        a.leaves = d.staged ? d.leafmask : nullptr;
        a.nleaf = d.staged ? N : 0;
        a.rstride = d.rstride;
        a.ring = kRing;
        a.nops = 0;
        a.nslot = d.nslot_cap;
        a.tile = tile;
        a.tpp = tpp;
        a.ppt = ppt;
        a.kact = K;
        a.npat = d.npat;
        a.ppad = d.ppad;
        a.root_last = 1;
        a.freqs = dfreq;
        a.partial = partial + (size_t)c * d.ntiles * 2;
        a.ticket = (unsigned *)(d.results + (size_t)c * 32);
        a.ninf = (uint32_t *)(d.results + (size_t)c * 32 + 4);
        a.err = (uint32_t *)(d.results + (size_t)c * 32 + 8);
        a.total = (double *)(d.results + (size_t)c * 32 + 16);
        a.ltab = d.ltab + (cfg->precision == CXG_FP64 ? (size_t)c * d.maxkids * 16 * K * 4 : 0);
        a.ntiles = d.ntiles;
        a.no_root = 0;
        jobs[c] = a;
    }
    for (unsigned t = 0; t < d.ntiles; ++t)
        for (unsigned c = 0; c < C; ++c) items.push_back(WalkItem{c, t});
    WalkItem *ditems = nullptr;
    e = cudaMemcpy(d.jobs, jobs.data(), C * sizeof(PlanArgs), cudaMemcpyHostToDevice);
    if (e != cudaSuccess || (rc = mc3_upload(h, &ditems, items.data(), items.size()))) {
        mc3_free(h);
        return rc ? rc : cuda_fail(e, "cudaMemcpy(jobs)");
    }
    BatchArgs &ba = h->ba;
    ba.jobs = d.jobs;
    ba.items = ditems;
    ba.nitems = (uint32_t)items.size();
    ba.counter = d.counter;
    ba.tile = tile;
    ba.tpp = tpp;
    ba.ppt = ppt;
    ba.ring = kRing;
    ba.kact = K;
    ba.max_nslot = d.nslot_cap;
    ba.max_rstride = d.rstride;
    ba.max_lmax = d.staged ? 0 : 3;
    ba.max_nleaf = d.staged ? N : 0;
    const size_t smem = plan_smem_bytes(cfg->precision, K, tile, d.nslot_cap, kRing,
                                        d.rstride, ba.max_lmax, ba.max_nleaf);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int per =
        batch_ctas_per_sm(cfg->precision, K, tile, tpp, ppt, d.staged != 0, smem);
    if (per <= 0) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: walker does not fit an SM");
    }
    h->grid = (unsigned)(per * nsm);
    h->pmat_grid = (C * d.maxkids * K + 31) / 32;
    h->propose_smem = mc3_propose_smem(NN, M);
    {  // (the default limit counts the kernel's static shared memory too)
        e = raise_propose_smem(h->propose_smem);
        if (e != cudaSuccess) {
            mc3_free(h);
            return cuda_fail(e, "cxgMc3Create: proposal shared memory");
        }
    }
    // Derived model quantities, then generation 0 (full evaluation).
    mc3_init_kernel<<<C, 32, 0, h->stream>>>(d);
    if ((e = cudaGetLastError()) != cudaSuccess) {
        mc3_free(h);
        return cuda_fail(e, "mc3_init_kernel");
    }
    if ((rc = mc3_enqueue_gen(h))) {
        mc3_free(h);
        return rc;
    }
    uint32_t st = 0;
    if ((e = cudaMemcpyAsync(&st, d.status, 4, cudaMemcpyDeviceToHost, h->stream)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) {
        mc3_free(h);
        return cuda_fail(e, "cxgMc3Create init");
    }
    if (st) {
        mc3_free(h);
        return fail(CXG_EINVAL, "cxgMc3Create: initial model cannot be decomposed");
    }
    // Capture a block of generations as one graph.
    h->graph_gens = cfg->graph_gens ? cfg->graph_gens : 16;
    cudaGraph_t graph = nullptr;
    {
        std::lock_guard<std::mutex> gate(capture_gate());
        e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (unsigned i = 0; i < h->graph_gens && rc == 0; ++i) rc = mc3_enqueue_gen(h);
            e = cudaStreamEndCapture(h->stream, &graph);
        }
    }
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        mc3_free(h);
        return rc ? rc : cuda_fail(e, "cudaStreamEndCapture(mc3)");
    }
    h->graph = graph;
    if ((e = cudaGraphInstantiate(&h->exec, graph, 0)) != cudaSuccess) {
        mc3_free(h);
        return cuda_fail(e, "cudaGraphInstantiate(mc3)");
    }
    *out = h;
    return 0;
}

extern "C" int cxgMc3Run(cxgMc3 *h, unsigned long long ngen, double *seconds) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgMc3Run: NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    NvtxRange nr("cxgMc3Run");
    cudaEvent_t t0, t1;
    CXG_CUDA(cudaEventCreate(&t0));
    CXG_CUDA(cudaEventCreate(&t1));
    CXG_CUDA(cudaEventRecord(t0, h->stream));
    unsigned long long left = ngen;
    while (left >= h->graph_gens) {
        CXG_CUDA(cudaGraphLaunch(h->exec, h->stream));
        left -= h->graph_gens;
    }
    for (; left > 0; --left) {
        int rc = mc3_enqueue_gen(h);
        if (rc) return rc;
    }
    CXG_CUDA(cudaEventRecord(t1, h->stream));
    CXG_CUDA(cudaEventSynchronize(t1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (seconds) *seconds = ms / 1e3;
    uint32_t st = 0;
    std::vector<char> res((size_t)h->d.nchains * 32);
    CXG_CUDA(cudaMemcpyAsync(&st, h->d.status, 4, cudaMemcpyDeviceToHost, h->stream));
    CXG_CUDA(cudaMemcpyAsync(res.data(), h->d.results, res.size(), cudaMemcpyDeviceToHost,
                             h->stream));
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    // Undecomposable proposed models are rejected, not errors (bit 0 is
    // only set for the initial model); bit 1 is a tree the eTBR re-rooting
    // could not walk, which a binary tree never gives.
    if (st & 2u) return fail(CXG_EINVAL, "MC3: an eTBR move met a malformed tree");
    // Any bounded wait that gave up?
    for (unsigned c = 0; c < h->d.nchains; ++c)
        if (*(const uint32_t *)(res.data() + (size_t)c * 32 + 8))
            return fail(CXG_ETIMEOUT, "MC3 walker: a record copy timed out");
    return 0;
}

int cxg::mc3_cold_lnl(cxgMc3 *h, double *out) {
    if (h == nullptr || out == nullptr) return fail(CXG_EINVAL, "mc3_cold_lnl: NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    const unsigned C = h->d.nchains;
    std::vector<double> v(2 * (size_t)C);
    CXG_CUDA(cudaMemcpyAsync(v.data(), h->d.lnL, C * 8, cudaMemcpyDeviceToHost, h->stream));
    CXG_CUDA(cudaMemcpyAsync(v.data() + C, h->d.heat, C * 8, cudaMemcpyDeviceToHost,
                             h->stream));
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    double best = -INFINITY;
    for (unsigned c = 0; c < C; ++c)
        if (v[C + c] == 1.0) best = v[c];
    *out = best;
    return 0;
}

extern "C" int cxgMc3Chain(cxgMc3 *h, unsigned chain, double *lnL, double *heat,
                           int32_t *parent, double *len, double *rates,
                           double *freqs, double *alpha) {
    if (h == nullptr || chain >= h->d.nchains) return fail(CXG_EINVAL, "cxgMc3Chain: bad chain");
    std::lock_guard<std::mutex> lk(h->mu);
    const Mc3Dev &d = h->d;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    if (lnL) CXG_CUDA(cudaMemcpy(lnL, d.lnL + chain, 8, cudaMemcpyDeviceToHost));
    if (heat) CXG_CUDA(cudaMemcpy(heat, d.heat + chain, 8, cudaMemcpyDeviceToHost));
    uint8_t tb = 0;
    CXG_CUDA(cudaMemcpy(&tb, d.curtree + chain, 1, cudaMemcpyDeviceToHost));
    const size_t t = (size_t)tb * d.nchains + chain;
    if (parent)
        CXG_CUDA(cudaMemcpy(parent, d.parent + t * d.nnodes, d.nnodes * 4,
                            cudaMemcpyDeviceToHost));
    if (len)
        CXG_CUDA(cudaMemcpy(len, d.len + t * d.nnodes, d.nnodes * 8,
                            cudaMemcpyDeviceToHost));
    uint8_t cm = 0;
    CXG_CUDA(cudaMemcpy(&cm, d.curmodel + chain, 1, cudaMemcpyDeviceToHost));
    Mc3Model m;
    CXG_CUDA(cudaMemcpy(&m, d.model + chain * 2 + cm, sizeof(m), cudaMemcpyDeviceToHost));
    const Mc3Sub &q = m.q[0];
    if (rates) memcpy(rates, q.rates, 48);
    if (freqs) memcpy(freqs, q.freqs, 32);
    // Gamma rates switched off read as the reference's alpha = INFINITY.
    if (alpha) *alpha = (d.ncat > 1 && !q.gamma_on) ? INFINITY : q.alpha;
    return 0;
}

// Checkpoint and resume.  A chain's state is its tree, heat and mixture
// members (cxgMc3Chain, cxgMc3ChainModel); with the generation count and
// the move counts it is all that a run carries from one generation to the
// next, since every draw comes from Philox keyed by (seed, chain,
// generation).  CLs are not saved: cxgMc3Resume recomputes them.

// Chain `chain` takes this tree (rooted at the run's root), heat and
// mixture.  Call cxgMc3Resume before running.
extern "C" int cxgMc3SetChain(cxgMc3 *h, unsigned chain, const int32_t *parent,
                              const double *len, const uint8_t *collapsed, double heat,
                              unsigned nmodels, const cxgMc3ModelState *models) {
    if (h == nullptr || chain >= h->d.nchains || parent == nullptr || len == nullptr ||
        models == nullptr)
        return fail(CXG_EINVAL, "cxgMc3SetChain: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    Mc3Dev &d = h->d;
    const unsigned N = d.ntaxa, NN = d.nnodes;
    if (nmodels < 1 || nmodels > d.mmax)
        return fail(CXG_EINVAL, "cxgMc3SetChain: 1..max_models members");
    if (!(heat > 0.0 && heat <= 1.0)) return fail(CXG_EINVAL, "cxgMc3SetChain: heat in (0, 1]");
    std::vector<int32_t> child(NN * 3, -1);
    std::vector<int> nch(NN, 0);
    for (unsigned v = 0; v < NN; ++v) {
        const int p = parent[v];
        if (v == d.root) {
            if (p != -1) return fail(CXG_EINVAL, "cxgMc3SetChain: root has a parent");
            continue;
        }
        if (p < (int)N || p >= (int)NN || nch[p] >= 3)
            return fail(CXG_EINVAL, "cxgMc3SetChain: not a binary tree at the run's root");
        if (!(len[v] >= 0.0)) return fail(CXG_EINVAL, "cxgMc3SetChain: negative length");
        child[p * 3 + nch[p]++] = (int)v;
    }
    for (unsigned v = N; v < NN; ++v)
        if (nch[v] != (v == d.root ? 3 : 2))
            return fail(CXG_EINVAL, "cxgMc3SetChain: tree is not binary (root degree 3)");
    std::vector<uint8_t> coll(NN, 0);
    if (collapsed)
        for (unsigned v = 0; v < NN; ++v) {
            if (!collapsed[v]) continue;
            if (v < N || v == d.root || len[v] != 0.0)
                return fail(CXG_EINVAL,
                            "cxgMc3SetChain: only internal edges of length 0 can be contracted");
            // (Only a run with polytomy jumps keeps its moves off them.)
            if (!d.poly)
                return fail(CXG_EINVAL, "cxgMc3SetChain: contracted edges need polytomy jumps");
            coll[v] = 1;
        }
    Mc3Model m;
    memset(&m, 0, sizeof(m));
    m.nmodels = (int32_t)nmodels;
    for (unsigned k = 0; k < nmodels; ++k) {
        const cxgMc3ModelState &s = models[k];
        Mc3Sub &q = m.q[k];
        int nr = 0;
        for (int i = 0; i < 6; ++i) {
            const int r = s.rclass[i];
            if (r < 0 || r > nr) return fail(CXG_EINVAL, "cxgMc3SetChain: rclass is not an RGS");
            if (r == nr) ++nr;
            for (int j = 0; j < i; ++j)
                if (s.rclass[j] == r && s.rates[j] != s.rates[i])
                    return fail(CXG_EINVAL, "cxgMc3SetChain: rates of one class differ");
            if (!(s.rates[i] > 0.0)) return fail(CXG_EINVAL, "cxgMc3SetChain: rates must be > 0");
            q.rates[i] = s.rates[i];
            q.rclass[i] = r;
        }
        q.nrates = nr;
        for (int i = 0; i < 4; ++i) {
            if (!(s.freqs[i] > 0.0)) return fail(CXG_EINVAL, "cxgMc3SetChain: freqs must be > 0");
            q.freqs[i] = s.freqs[i];
        }
        q.freqs_est = s.freqs_est ? 1 : 0;
        if (!q.freqs_est && !(q.freqs[0] == q.freqs[1] && q.freqs[1] == q.freqs[2] &&
                              q.freqs[2] == q.freqs[3]))
            return fail(CXG_EINVAL, "cxgMc3SetChain: equal-frequency member with unequal freqs");
        q.gamma_on = (d.ncat > 1 && !isinf(s.alpha)) ? 1 : 0;
        q.alpha = isinf(s.alpha) ? 1.0 : s.alpha;
        if (q.gamma_on && !(q.alpha > 0.0)) return fail(CXG_EINVAL, "cxgMc3SetChain: alpha");
        q.wvar = d.invar ? s.wvar : 1.0;
        q.winvar = d.invar ? s.winvar : 0.0;
        q.weight = s.weight;
        q.rmult = s.rmult;
        if (!(q.wvar > 0.0 && q.winvar >= 0.0 && q.weight > 0.0 && q.rmult > 0.0))
            return fail(CXG_EINVAL, "cxgMc3SetChain: weights must be positive");
    }
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    const size_t t0 = (size_t)0 * d.nchains + chain, t1 = (size_t)1 * d.nchains + chain;
    for (size_t t : {t0, t1}) {
        CXG_CUDA(cudaMemcpy(d.parent + t * NN, parent, NN * 4, cudaMemcpyHostToDevice));
        CXG_CUDA(cudaMemcpy(d.child + t * NN * 3, child.data(), NN * 12, cudaMemcpyHostToDevice));
        CXG_CUDA(cudaMemcpy(d.len + t * NN, len, NN * 8, cudaMemcpyHostToDevice));
        CXG_CUDA(cudaMemcpy(d.coll + t * NN, coll.data(), NN, cudaMemcpyHostToDevice));
    }

    const uint8_t zero = 0;
    const int32_t none = 0;
    CXG_CUDA(cudaMemcpy(d.fl_nd + chain, &none, 4, cudaMemcpyHostToDevice));
    CXG_CUDA(cudaMemcpy(d.curtree + chain, &zero, 1, cudaMemcpyHostToDevice));
    CXG_CUDA(cudaMemcpy(d.curmodel + chain, &zero, 1, cudaMemcpyHostToDevice));
    CXG_CUDA(cudaMemcpy(d.model + (size_t)chain * 2, &m, sizeof(m), cudaMemcpyHostToDevice));
    CXG_CUDA(cudaMemcpy(d.heat + chain, &heat, 8, cudaMemcpyHostToDevice));
    return 0;
}

// Per-chain accept and reject counts ([chain][move], kMoves moves) and
// swap counts, as cxgMc3Stats gives them.
extern "C" int cxgMc3SetCounts(cxgMc3 *h, const unsigned *accepts, const unsigned *rejects,
                               const unsigned *swaps) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgMc3SetCounts: NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    const Mc3Dev &d = h->d;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    if (accepts)
        CXG_CUDA(cudaMemcpy(d.acc, accepts, (size_t)d.nchains * kMoves * 4,
                            cudaMemcpyHostToDevice));
    if (rejects)
        CXG_CUDA(cudaMemcpy(d.rej, rejects, (size_t)d.nchains * kMoves * 4,
                            cudaMemcpyHostToDevice));
    if (swaps) CXG_CUDA(cudaMemcpy(d.nswap, swaps, d.nchains * 4, cudaMemcpyHostToDevice));
    return 0;
}

// Recompute every chain's CLs and lnL from its tree and mixture (a full
// evaluation, as generation 0 does), then continue at `generation`: the
// next generation draws what an uninterrupted run draws there.
extern "C" int cxgMc3Resume(cxgMc3 *h, unsigned long long generation) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgMc3Resume: NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    Mc3Dev &d = h->d;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    // No previous move to flip in; generation 0 is the full evaluation.
    std::vector<Mc3Prop> props(d.nchains);
    memset(props.data(), 0, props.size() * sizeof(Mc3Prop));
    CXG_CUDA(cudaMemcpy(d.prop, props.data(), props.size() * sizeof(Mc3Prop),
                        cudaMemcpyHostToDevice));
    const unsigned long long g0 = 0;
    CXG_CUDA(cudaMemcpy(d.gen, &g0, 8, cudaMemcpyHostToDevice));
    const uint32_t st0 = 0;
    CXG_CUDA(cudaMemcpy(d.status, &st0, 4, cudaMemcpyHostToDevice));
    mc3_init_kernel<<<d.nchains, 32, 0, h->stream>>>(d);
    CXG_CHECK_LAUNCH("mc3_init_kernel");
    int rc = mc3_enqueue_gen(h);
    if (rc) return rc;
    uint32_t st = 0;
    CXG_CUDA(cudaMemcpyAsync(&st, d.status, 4, cudaMemcpyDeviceToHost, h->stream));
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    if (st & 1u) return fail(CXG_EINVAL, "cxgMc3Resume: a model cannot be decomposed");
    std::vector<char> res((size_t)d.nchains * 32);
    CXG_CUDA(cudaMemcpy(res.data(), d.results, res.size(), cudaMemcpyDeviceToHost));
    for (unsigned c = 0; c < d.nchains; ++c)
        if (*(const uint32_t *)(res.data() + (size_t)c * 32 + 8))
            return fail(CXG_ETIMEOUT, "MC3 walker: a record copy timed out");
    CXG_CUDA(cudaMemcpy(d.gen, &generation, 8, cudaMemcpyHostToDevice));
    return 0;
}

extern "C" int cxgMc3ChainCollapsed(cxgMc3 *h, unsigned chain, uint8_t *out) {
    if (h == nullptr || chain >= h->d.nchains || out == nullptr)
        return fail(CXG_EINVAL, "cxgMc3ChainCollapsed: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    const Mc3Dev &d = h->d;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    uint8_t tb = 0;
    CXG_CUDA(cudaMemcpy(&tb, d.curtree + chain, 1, cudaMemcpyDeviceToHost));
    const size_t t = (size_t)tb * d.nchains + chain;
    CXG_CUDA(cudaMemcpy(out, d.coll + t * d.nnodes, d.nnodes, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int cxgMc3ChainModel(cxgMc3 *h, unsigned chain, unsigned model,
                                unsigned *nmodels, cxgMc3ModelState *out) {
    if (h == nullptr || chain >= h->d.nchains || model >= (unsigned)kMaxModels)
        return fail(CXG_EINVAL, "cxgMc3ChainModel: bad chain or model");
    std::lock_guard<std::mutex> lk(h->mu);
    const Mc3Dev &d = h->d;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    uint8_t cm = 0;
    CXG_CUDA(cudaMemcpy(&cm, d.curmodel + chain, 1, cudaMemcpyDeviceToHost));
    Mc3Model m;
    CXG_CUDA(cudaMemcpy(&m, d.model + chain * 2 + cm, sizeof(m), cudaMemcpyDeviceToHost));
    if (nmodels) *nmodels = (unsigned)m.nmodels;
    if (out == nullptr) return 0;
    if ((int)model >= m.nmodels) return fail(CXG_EINVAL, "cxgMc3ChainModel: no such model");
    const Mc3Sub &q = m.q[model];
    memcpy(out->rates, q.rates, 48);
    memcpy(out->freqs, q.freqs, 32);
    out->alpha = (d.ncat > 1 && !q.gamma_on) ? INFINITY : q.alpha;
    out->wvar = q.wvar;
    out->winvar = q.winvar;
    out->weight = q.weight;
    out->rmult = q.rmult;
    for (int i = 0; i < 6; ++i) out->rclass[i] = q.rclass[i];
    out->nrates = q.nrates;
    out->freqs_est = q.freqs_est;
    return 0;
}

extern "C" int cxgMc3ChainWeights(cxgMc3 *h, unsigned chain, double *wvar, double *winvar) {
    if (h == nullptr || chain >= h->d.nchains)
        return fail(CXG_EINVAL, "cxgMc3ChainWeights: bad chain");
    std::lock_guard<std::mutex> lk(h->mu);
    const Mc3Dev &d = h->d;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    uint8_t cm = 0;
    CXG_CUDA(cudaMemcpy(&cm, d.curmodel + chain, 1, cudaMemcpyDeviceToHost));
    Mc3Model m;
    CXG_CUDA(cudaMemcpy(&m, d.model + chain * 2 + cm, sizeof(m), cudaMemcpyDeviceToHost));
    if (wvar) *wvar = m.q[0].wvar;
    if (winvar) *winvar = m.q[0].winvar;
    return 0;
}

extern "C" int cxgMc3Stats(cxgMc3 *h, unsigned *accepts, unsigned *rejects,
                           unsigned *swaps, unsigned long long *gen) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgMc3Stats: NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    const Mc3Dev &d = h->d;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    if (accepts)
        CXG_CUDA(cudaMemcpy(accepts, d.acc, (size_t)d.nchains * kMoves * 4,
                            cudaMemcpyDeviceToHost));
    if (rejects)
        CXG_CUDA(cudaMemcpy(rejects, d.rej, (size_t)d.nchains * kMoves * 4,
                            cudaMemcpyDeviceToHost));
    if (swaps) CXG_CUDA(cudaMemcpy(swaps, d.nswap, d.nchains * 4, cudaMemcpyDeviceToHost));
    if (gen) CXG_CUDA(cudaMemcpy(gen, d.gen, 8, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int cxgMc3Trace(cxgMc3 *h, double *out, unsigned long long n) {
    if (h == nullptr) return fail(CXG_EINVAL, "cxgMc3Trace: NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    if (n > h->d.trace_cap) n = h->d.trace_cap;
    CXG_CUDA(cudaStreamSynchronize(h->stream));
    CXG_CUDA(cudaMemcpy(out, h->d.trace, n * 8, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int cxgMc3Destroy(cxgMc3 *h) {
    if (h == nullptr) return 0;
    {
        std::lock_guard<std::mutex> lk(h->mu);  // waits for a call in progress
        cudaStreamSynchronize(h->stream);
    }
    mc3_free(h);
    return 0;
}
