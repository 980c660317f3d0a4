// cxgPlanSnapRun: the step planner of Lik._plan / Lik._planRecurse
// (pkg/Crux/Tree/Lik.pyx:1427-1601) over a flattened rooted traversal.
//
// The host mirror (crux_gb300/lik.py) flattens the tree once per topology,
// root and set of CL buffers into visits in the planner's post-order.  This
// file then does per evaluation what the recursion does per node, in the same
// order, so the step array, the CxtLikCL fields and the valid flags come out
// exactly as the Python restatement leaves them:
//
//   1. a CL whose parent, nSibs or edge length changed (or every CL when the
//      Lik is invalidated) marks its parent dirty and takes the new values
//      (Lik.pyx:1492-1502);
//   2. a dirty internal CL gets one Compute step and degree-2 Merge steps,
//      one per child in ring order, with ntrail counting down to 0, and
//      marks its parent dirty (Lik.pyx:1504-1530);
//   3. the root CL gets the same over all of its children (Lik.pyx:1560-1597);
//   4. every visited CL's struct valid flag is brought up to date.
//
// Host code only: no CUDA call is made here.
#include <stdint.h>
#include <string.h>

#include <vector>

#include "cxg_internal.h"

namespace {

inline double length_of(const double *lens, int32_t e) {
    return e < 0 ? 0.0 : lens[e];
}

}  // namespace

extern "C" int cxgPlanSnapRun(const cxgPlanSnap *s, const double *lens,
                              int invalidate, CxtLikStep *steps, uint32_t cap,
                              uint32_t *nsteps, uint32_t *changed,
                              uint32_t *nchanged) {
    using cxg::fail;
    if (s == nullptr || nsteps == nullptr || changed == nullptr ||
        nchanged == nullptr || (cap != 0 && steps == nullptr))
        return fail(CXG_EINVAL, "cxgPlanSnapRun: NULL argument");
    const uint32_t nvis = s->nvis;
    *nsteps = 0;
    *nchanged = 0;
    if (nvis == 0 || s->up[nvis - 1] >= 0)
        return fail(CXG_EINVAL, "cxgPlanSnapRun: the last visit must be the root");
    // mark[v]: visit v's mirrors differ from what the caller holds; valid0
    // keeps the valid flags as they came in (a CL marked dirty and then
    // recomputed in this plan ends where it began).
    static thread_local std::vector<uint8_t> mark, valid0;
    mark.assign(nvis, 0);
    valid0.assign(s->valid, s->valid + nvis);
    const bool inval = invalidate != 0;
    uint32_t ns = 0;
    int status = 0;

    for (uint32_t v = 0; v < nvis && status == 0; ++v) {
        CxtLikCL *cl = s->cl[v];
        const int32_t up = s->up[v];
        if (up >= 0) {
            if ((uint32_t)up <= v || (uint32_t)up >= nvis)
                return fail(CXG_EINVAL, "cxgPlanSnapRun: parent visit out of order");
            CxtLikCL *par = s->cl[up];
            const double el = length_of(lens, s->edge[v]);
            const uint32_t nsib = s->nsibs[v];
            if (inval || s->m_parent[v] != par || s->m_nsibs[v] != nsib ||
                s->m_elen[v] != el) {
                s->valid[up] = 0;
                if (s->m_parent[v] != par) {
                    s->m_parent[v] = par;
                    cl->parent = par;
                    mark[v] = 1;
                }
                if (s->m_nsibs[v] != nsib) {
                    s->m_nsibs[v] = nsib;
                    cl->nSibs = nsib;
                    mark[v] = 1;
                }
                if (s->m_elen[v] != el) {
                    s->m_elen[v] = el;
                    cl->edgeLen = el;
                    mark[v] = 1;
                }
            }
        }
        const uint32_t nk = s->nkids[v];
        if (nk == 0) continue;  // a leaf
        if (!(inval || !s->valid[v])) continue;
        if (nk == 1 && up >= 0)
            return fail(CXG_EINVAL, "cxgPlanSnapRun: internal node of degree 2");
        const uint32_t k0 = s->kid0[v];
        if (k0 + nk > s->nkid || k0 + nk < k0)
            return fail(CXG_EINVAL, "cxgPlanSnapRun: child range out of bounds");
        if (ns + nk > cap)
            return fail(CXG_EINVAL, "cxgPlanSnapRun: step array is full");
        for (uint32_t j = 0; j < nk; ++j) {
            const uint32_t c = k0 + j;
            const double el = length_of(lens, s->kid_edge[c]);
            if (el < 0.0) {
                status = 1;  // ValueError("Negative branch length")
                break;
            }
            CxtLikStep &st = steps[ns + j];
            st.variant = s->kid_int[c]
                             ? (j == 0 ? CxeLikStepComputeI : CxeLikStepMergeI)
                             : (j == 0 ? CxeLikStepComputeL : CxeLikStepMergeL);
            st.ntrail = nk - 1 - j;
            st.parentCL = cl;
            st.childCL = s->kid_cl[c];
            st.edgeLen = el;
        }
        if (status) break;
        ns += nk;
        s->valid[v] = 1;
        if (up >= 0) s->valid[up] = 0;
    }

    if (status == 0) {
        // Struct valid flags follow the mirrors (CL.sync_valid).
        for (uint32_t v = 0; v < nvis; ++v) {
            if (s->cvalid[v] != s->valid[v]) {
                s->cl[v]->valid = s->valid[v] != 0;
                s->cvalid[v] = s->valid[v];
                mark[v] = 1;
            }
        }
        *nsteps = ns;
    }
    uint32_t nc = 0;
    for (uint32_t v = 0; v < nvis; ++v)
        if (mark[v] || s->valid[v] != valid0[v]) changed[nc++] = v;
    *nchanged = nc;
    return status;
}
