/* integration_example.c -- the C usage of libhydrocuda that the integration
 * notes show (a solver's lifecycle, a batch's admission, stepping and fetch),
 * as one function; tests/test_abi.py compiles it against include/hydrocuda.h. */
#include <stdio.h>
#include <stddef.h>
#include "hydrocuda.h"

void example(double* cons_aos6, int count, const hc_solver_desc* descs, const void* const* states,
             const long long* max_steps, void** results) {
hc_context* ctx; hc_solver* s;
hc_solver_desc d = {0};
d.dim = 1; d.n[0] = 256; d.mins[0] = -1; d.maxs[0] = 1;
for (int k = 0; k < 6; ++k) d.boundary[k] = HC_BOUNDARY_FREEFLOW;
d.flux_limiter = HC_LIMITER_SUPERBEE; d.recon = HC_RECON_NONE;
d.integrator = HC_INT_FORWARD_EULER; d.precision = HC_F64_PLAIN;
d.gamma = 1.4; d.rho_min = 1e-7; d.p_min = 1e-7; d.cfl = .5;
hc_context_create(0, &ctx);
if (hc_solver_create(ctx, &d, &s) != HC_OK) puts(hc_last_error());
hc_solver_reset_state(s, cons_aos6, HC_LAYOUT_AOS6_F64);
long long n; hc_solver_run_until(s, 0.2, 1LL << 40, &n);
hc_solver_get_state(s, cons_aos6, HC_LAYOUT_AOS6_F64, 0);
hc_batch_desc bd = {0};
bd.precision = HC_F32_FUSED; bd.max_slots = 512; bd.hbm_budget = (size_t)64 << 30;
bd.recon = HC_RECON_PLM_CONS; bd.slope_limiter = HC_LIMITER_VAN_LEER_ABS;
bd.integrator = HC_INT_RK2; bd.flux = HC_FLUX_ROE;
hc_batch* b; hc_batch_create(ctx, &bd, &b);
int slots[512], got;
if (hc_batch_admit_many(b, count, descs, states, HC_LAYOUT_SOA5_F32, NULL, max_steps, NULL,
                        slots, &got) != HC_OK)
    puts(hc_last_error());                     /* the first `got` are admitted */
int active;
do hc_batch_step(b, 8, &active); while (active > 0);
hc_done done[512]; int nd;
hc_batch_poll(b, done, 512, &nd);              /* tag = admission index when tags is NULL */
int fs[512]; void* outs[512];
for (int k = 0; k < nd; ++k) { fs[k] = done[k].slot; outs[k] = results[done[k].tag]; }
hc_batch_fetch_many(b, nd, fs, outs, HC_LAYOUT_SOA5_F32);
}
