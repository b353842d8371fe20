// hc_plan.cu -- Runge-Kutta tables and their fused-stage plans (host only).
#include "hc_internal.h"

#include <cstring>

namespace hc {

// hydro/int/all.lua:10-155; index 0 is forward Euler (hydro/int/fe.lua).
static const RKTable kTables[HC_NUM_INTEGRATORS] = {
    {1, {{1}}, {{1}}},
    {2, {{1, 0}, {1, 0}}, {{.5, 0}, {0, 1}}},
    {2, {{1, 0}, {1, 0}}, {{1, 0}, {.5, .5}}},
    {2, {{1, 0}, {1, 0}}, {{2. / 3., 0}, {1. / 4., 3. / 4.}}},
    {3, {{1, 0, 0}, {1, 0, 0}, {1, 0, 0}}, {{.5, 0, 0}, {-1, 2, 0}, {1. / 6., 2. / 6., 1. / 6.}}},
    {4, {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}},
        {{.5, 0, 0, 0}, {0, .5, 0, 0}, {0, 0, 1, 0}, {1. / 6., 2. / 6., 2. / 6., 1. / 6.}}},
    {4, {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}},
        {{1. / 3., 0, 0, 0}, {-1. / 3., 0, 0, 0}, {1, -1, 1, 0}, {1. / 8., 3. / 8., 3. / 8., 1. / 8.}}},
    {2, {{1, 0}, {.5, .5}}, {{1, 0}, {0, .5}}},
    {2, {{1, 0}, {1, 0}}, {{-20, 0}, {41. / 40., -1. / 40.}}},
    {3, {{1, 0, 0}, {3. / 4., 1. / 4., 0}, {1. / 3., 0, 2. / 3.}}, {{1, 0, 0}, {0, 1. / 4., 0}, {0, 0, 2. / 3.}}},
    {4, {{1, 0, 0, 0}, {649. / 1600., 951. / 1600., 0, 0}, {53989. / 2500000., 4806213. / 20000000., 23619. / 32000., 0},
         {1. / 5., 6127. / 30000., 7873. / 30000., 1. / 3.}},
        {{.5, 0, 0, 0}, {-10890423. / 25193600., 5000. / 7873, 0, 0}, {-102261. / 5000000., -5121. / 20000., 7873. / 10000., 0},
         {1. / 10., 1. / 6., 0, 1. / 6.}}},
    {4, {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {-1. / 3., 1. / 3., 2. / 3., 1. / 3.}},
        {{.5, 0, 0, 0}, {0, .5, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1. / 6.}}},
};

const RKTable& rk_table(int integrator) { return kTables[integrator]; }

// Stage s (1-based) produces u^(s+1) from u^(s) (read with its halo), the
// states u^(k) (k <= s, pointwise) and the derivatives L(u^(k)) (k < s
// stored, k = s computed in the same launch).  The output buffer may reuse a
// buffer whose only remaining read is pointwise in this very stage; the last
// stage prefers buffer 0 so the state stays in place whenever the table
// allows it.
IntegratorPlan make_plan(int integrator) {
    const RKTable& T = kTables[integrator];
    int const order = T.order;
    IntegratorPlan P;
    std::memset(&P, 0, sizeof(P));
    P.n_stages = order;

    // last stage (1-based s) that reads u^(k) pointwise; halo use is stage k
    auto lastUseState = [&](int k) {
        int last = k;  // the halo read in stage k
        for (int s = k; s <= order; ++s)
            if (T.alpha[s - 1][k - 1] != 0) last = s > last ? s : last;
        return last;
    };
    auto lastUseDeriv = [&](int k) {
        int last = 0;
        for (int s = k + 1; s <= order; ++s)
            if (T.beta[s - 1][k - 1] != 0) last = s;
        return last;
    };

    int stateBuf[6];      // buffer holding u^(k)
    int bufOwner[8];      // which u^(k) a state buffer holds (0 = free)
    for (int b = 0; b < 8; ++b) bufOwner[b] = 0;
    stateBuf[1] = 0;
    bufOwner[0] = 1;
    int nState = 1;
    int derivBuf[6];
    int derivOwner[8];
    for (int b = 0; b < 8; ++b) derivOwner[b] = 0;
    int nDeriv = 0;

    for (int s = 1; s <= order; ++s) {
        StagePlan& S = P.stage[s - 1];
        S.index = s - 1;
        S.in_buf = stateBuf[s];
        S.n_alpha = 0;
        for (int k = 1; k <= s; ++k)
            if (T.alpha[s - 1][k - 1] != 0) {
                S.alpha[S.n_alpha].buf = stateBuf[k];
                S.alpha[S.n_alpha].coef = T.alpha[s - 1][k - 1];
                S.n_alpha++;
            }
        S.n_beta = 0;
        for (int k = 1; k < s; ++k)
            if (T.beta[s - 1][k - 1] != 0) {
                S.beta[S.n_beta].buf = derivBuf[k];
                S.beta[S.n_beta].coef = T.beta[s - 1][k - 1];
                S.n_beta++;
            }
        S.beta_cur = T.beta[s - 1][s - 1];
        S.last = s == order;
        // store L(u^(s)) if a later stage needs it
        S.store_deriv = -1;
        if (lastUseDeriv(s) > s) {
            int b = -1;
            for (int c = 0; c < 8 && b < 0; ++c)
                if (derivOwner[c] == 0 || lastUseDeriv(derivOwner[c]) < s) b = c;
            derivOwner[b] = s;
            derivBuf[s] = b;
            if (b + 1 > nDeriv) nDeriv = b + 1;
            S.store_deriv = b;
        }
        // output buffer: not the halo input; any other buffer whose state is
        // not needed after this stage
        auto usable = [&](int b) {
            if (b == S.in_buf) return false;
            int const k = bufOwner[b];
            if (k == 0) return true;
            return lastUseState(k) <= s;
        };
        int out = -1;
        if (S.last && usable(0)) out = 0;
        for (int b = 0; b < 8 && out < 0; ++b)
            if (usable(b)) out = b;
        S.out_buf = out;
        bufOwner[out] = s + 1;
        stateBuf[s + 1] = out;
        if (out + 1 > nState) nState = out + 1;
    }
    P.n_state_bufs = nState;
    P.n_deriv_bufs = nDeriv;
    P.result_buf = stateBuf[order + 1];
    return P;
}

}  // namespace hc
