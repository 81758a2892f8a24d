/*
 * or_step.c — TEST INFRASTRUCTURE (the oracle).  FP64 time stepping around the BGC functors:
 *  - BoxModel RK3 (src/BoxModel/timesteppers.jl:30-93): U += dt*(gamma*G + zeta*G-), with
 *    Oceananigans' RungeKutta3 coefficients gamma = (8/15, 5/12, 3/4), zeta = (-, -17/60, -5/12)
 *    and stage times t, t + 8/15 dt, t + 2/3 dt.
 *  - 3-D tracer step: flux-form WENO5 advection by the model velocity and by each tracer's drift
 *    velocity (Oceananigans div_Uc; restated from the published WENO-Z scheme of Borges et al.
 *    2008 with p = 2 and eps = 1e-8, order reduced to WENO3 and first-order upwind next to Bounded
 *    walls), the BGC functors, TwoBand PAR recomputed from the state at every stage
 *    (update_biogeochemical_state! after every substep), RK3.  Parity with Oceananigans itself is
 *    unpinned (it is not in this container).
 *  - Columns with vertically implicit diffusion after every explicit substep (Oceananigans
 *    VerticallyImplicitTimeDiscretization, stage dt = (gamma + zeta) dt), zero-flux walls.
 *  - ScaleNegativeTracers (src/Utils/negative_tracers.jl:250-276).
 */
#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include "obgc_oracle.h"

static const double RK_G[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};
static const double RK_Z[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
static const double RK_C[3] = {0.0, 8.0 / 15.0, 2.0 / 3.0};

/* splitmix64 finaliser: the sign source of the conditioning probe (or_model3d.stage_rounding) */
static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* ------------------------------------------------------------------ WENO ---------- */
static double weno5(double v1, double v2, double v3, double v4, double v5) {
    const double eps = 1e-8;
    double q0 = (2 * v1 - 7 * v2 + 11 * v3) / 6;
    double q1 = (-v2 + 5 * v3 + 2 * v4) / 6;
    double q2 = (2 * v3 + 5 * v4 - v5) / 6;
    double a = v1 - 2 * v2 + v3, b = v1 - 4 * v2 + 3 * v3;
    double b0 = 13.0 / 12.0 * a * a + 0.25 * b * b;
    a = v2 - 2 * v3 + v4; b = v2 - v4;
    double b1 = 13.0 / 12.0 * a * a + 0.25 * b * b;
    a = v3 - 2 * v4 + v5; b = 3 * v3 - 4 * v4 + v5;
    double b2 = 13.0 / 12.0 * a * a + 0.25 * b * b;
    double tau = fabs(b0 - b2);
    double r0 = tau / (b0 + eps), r1 = tau / (b1 + eps), r2 = tau / (b2 + eps);
    double a0 = 0.1 * (1 + r0 * r0), a1 = 0.6 * (1 + r1 * r1), a2 = 0.3 * (1 + r2 * r2);
    return (a0 * q0 + a1 * q1 + a2 * q2) / (a0 + a1 + a2);
}
static double weno3(double v1, double v2, double v3) {
    const double eps = 1e-8;
    double q0 = (-v1 + 3 * v2) / 2, q1 = (v2 + v3) / 2;
    double b0 = (v2 - v1) * (v2 - v1), b1 = (v3 - v2) * (v3 - v2);
    double tau = fabs(b0 - b1);
    double r0 = tau / (b0 + eps), r1 = tau / (b1 + eps);
    double a0 = (1.0 / 3.0) * (1 + r0 * r0), a1 = (2.0 / 3.0) * (1 + r1 * r1);
    return (a0 * q0 + a1 * q1) / (a0 + a1);
}

/* Upwind-biased value at face f (between cells f-1 and f) of a line of N cells with stride s. */
static double face_value(const double* c, long s, int N, int periodic, int f, double U) {
#define C(m) c[(long)(periodic ? (((m) % N) + N) % N : (m)) * s]
    if (periodic) {
        if (U > 0) return weno5(C(f - 3), C(f - 2), C(f - 1), C(f), C(f + 1));
        return weno5(C(f + 2), C(f + 1), C(f), C(f - 1), C(f - 2));
    }
    int b = f < N - f ? f : N - f;
    if (b == 0) return f == 0 ? C(0) : C(N - 1);
    if (b >= 3) {
        if (U > 0) return weno5(C(f - 3), C(f - 2), C(f - 1), C(f), C(f + 1));
        return weno5(C(f + 2), C(f + 1), C(f), C(f - 1), C(f - 2));
    }
    if (b == 2) {
        if (U > 0) return weno3(C(f - 2), C(f - 1), C(f));
        return weno3(C(f + 1), C(f), C(f - 1));
    }
    return U > 0 ? C(f - 1) : C(f);
#undef C
}

/* ------------------------------------------------------------------ box ---------- */
void or_box_run(const obgc_npd_params* p, double* v, const double* PAR_stages, double PAR_const,
                double t0, double dt, int nsteps) {
    int32_t names[32];
    int n = or_npd_required_tracers(p, names, 32);
    double G[OBGC_NUM_NAMED] = {0}, Gm[OBGC_NUM_NAMED] = {0};
    (void)t0;
    for (int s = 0; s < nsteps; s++) {
        for (int st = 0; st < 3; st++) {
            double PAR = PAR_stages ? PAR_stages[3 * s + st] : PAR_const;
            for (int q = 0; q < n; q++) G[names[q]] = or_npd_tendency(p, names[q], v, PAR);
            for (int q = 0; q < n; q++) {
                int nm = names[q];
                if (st == 0) v[nm] += dt * RK_G[0] * G[nm];
                else v[nm] += dt * (RK_G[st] * G[nm] + RK_Z[st] * Gm[nm]);
            }
            memcpy(Gm, G, sizeof(G));
        }
    }
}

/* BoxModel(; forcing, prescribed_tracers) (boxmodel.jl:65-87, timesteppers.jl:37-63): before
 * the tendencies of stage st of step s, update_state! sets each prescribed tracer to its value at
 * the stage time (row 3 s + st of presc[q]); after the step, to its value at the step's end (row
 * 3 (s + 1)).  A forcing adds its stage-time rate (row 3 s + st of frc[q]) to the tracer's
 * tendency.  presc[q]: [3 nsteps + 1], frc[q]: [3 nsteps]. */
void or_box_run_drivers(const obgc_npd_params* p, double* v, const double* PAR_stages, double PAR_const, double dt,
                        int nsteps, int np, const int32_t* pnames, const double* const* presc, int nf,
                        const int32_t* fnames, const double* const* frc) {
    int32_t names[32];
    int n = or_npd_required_tracers(p, names, 32);
    double G[OBGC_NUM_NAMED] = {0}, Gm[OBGC_NUM_NAMED] = {0};
    for (int s = 0; s < nsteps; s++) {
        for (int st = 0; st < 3; st++) {
            for (int q = 0; q < np; q++) v[pnames[q]] = presc[q][3 * s + st];
            double PAR = PAR_stages ? PAR_stages[3 * s + st] : PAR_const;
            for (int q = 0; q < n; q++) G[names[q]] = or_npd_tendency(p, names[q], v, PAR);
            for (int q = 0; q < nf; q++) G[fnames[q]] += frc[q][3 * s + st];
            for (int nm = 0; nm < OBGC_NUM_NAMED; nm++) {
                if (st == 0) v[nm] += dt * RK_G[0] * G[nm];
                else v[nm] += dt * (RK_G[st] * G[nm] + RK_Z[st] * Gm[nm]);
            }
            memcpy(Gm, G, sizeof(G));
            memset(G, 0, sizeof(G));
        }
        for (int q = 0; q < np; q++) v[pnames[q]] = presc[q][3 * (s + 1)];
    }
}

/* ------------------------------------------------------------------ 3-D ---------- */
static double surface_par(const or_model3d* m, double t) {
    return m->surface_kind == OBGC_SURFACE_PAR_CONSTANT ? m->surface_value : or_default_surface_PAR(t);
}

static int slot_of(const or_model3d* m, int name) {
    for (int q = 0; q < m->n_tracers; q++) if (m->names[q] == name) return q;
    return -1;
}

void or_par3d(const or_model3d* m, const double* state, double t, double* PAR, int nthreads) {
    const obgc_grid* g = &m->grid;
    int Nx = g->Nx, Ny = g->Ny, Nz = g->Nz;
    long NN = (long)Nx * Ny;
    double dz = g->Lz / Nz;
    double* zc = malloc(sizeof(double) * Nz);
    double* zf = malloc(sizeof(double) * (Nz + 1));
    for (int k = 0; k <= Nz; k++) zf[k] = -g->Lz + k * dz;
    for (int k = 0; k < Nz; k++) zc[k] = -g->Lz + (k + 0.5) * dz;
    int sP = slot_of(m, OBGC_P);
    double PAR0 = surface_par(m, t);
#pragma omp parallel num_threads(nthreads)
    {
        double* col = malloc(sizeof(double) * Nz);
        double* out = malloc(sizeof(double) * Nz);
#pragma omp for schedule(static)
        for (long c = 0; c < NN; c++) {
            for (int k = 0; k < Nz; k++) col[k] = state[(long)sP * NN * Nz + k * NN + c];
            or_twoband_column(&m->light, Nz, zc, zf, col, PAR0, out);
            for (int k = 0; k < Nz; k++) PAR[k * NN + c] = out[k];
        }
        free(col); free(out);
    }
    free(zc); free(zf);
}

/* update_biogeochemical_state!(model, ::ScaleNegativeTracers / ::ZeroNegativeTracers)
 * (negative_tracers.jl:23-29, :136-143) on every cell of a 3-D state. */
static void or_negatives3d(const or_model3d* m, double* state, long N, int ng, const int32_t* gn,
                           const int32_t* gslot, const double* gfac, int nthreads) {
    if (m->negatives == 1) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (long c = 0; c < N; c++) or_scale_cell(state + c, N, ng, gn, gslot, gfac, m->invalid_fill_value);
    } else if (m->negatives == 2) {
        for (int q = 0; q < m->n_tracers; q++) {
            if ((m->zero_exclude_mask >> q) & 1) continue;
            double* x = state + (long)q * N;
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (long c = 0; c < N; c++) x[c] = x[c] > 0.0 ? x[c] : (isnan(x[c]) ? x[c] : 0.0);
        }
    }
}

static void implicit_diffusion(int Nz, double dz, const double* kf, double dts, double* x, double* cp, double* dp);

/* ------------------------------------------------------------------ SimpleMultiG ---------- */
/* simple_multi_G.jl:163-189: the fields' tendencies from the deposited nitrogen flux */
static void or_mg_tendency(const obgc_multig_params* p, double Ns, double Nf, double flux, double G[3]) {
    G[0] = (1 - p->refactory_fraction) * p->slow_fraction * flux - p->slow_decay_rate * Ns;
    G[1] = (1 - p->refactory_fraction) * p->fast_fraction * flux - p->fast_decay_rate * Nf;
    G[2] = p->refactory_fraction * flux;
}

/* ifelse(isfinite(p), p, zero(Nr)) (simple_multi_G.jl:379,395,410).  A log of a negative argument
 * throws in Julia on the CPU and gives NaN on the GPU; here it is NaN, so the fraction is zero. */
static double or_mg_fraction(double p) { return isfinite(p) ? p : 0.0; }

/* simple_multi_G.jl:193-247 (NH4, NO3, O2 of the nitrogen-only form) with the fractions of
 * :352-426; F = (NO3, NH4, O2) in mmol / m2 / s */
static void or_mg_coupling(const obgc_multig_params* p, double Ns, double Nf, double NO3, double NH4, double O2,
                           double F[3]) {
    const double day = 86400.0, R = p->sinking_redfield, ls = p->slow_decay_rate, lf = p->fast_decay_rate;
    const double Nr = ls * Ns + lf * Nf;
    const double Cr = Nr * R;
    const double k = (ls * (Ns * R) + lf * (Nf * R)) / (Ns * R + Nf * R + DBL_TRUE_MIN);   /* reactivity */
    const double kO2 = p->anoxia_half_saturation;
    const double* A = p->nitrate_oxidation;
    const double pn = or_mg_fraction(exp(A[0] + A[1] * log(Cr * day) * log(O2) + A[2] * pow(log(Cr * day), 2) +
                                         A[3] * log(k * day) * log(NH4) + A[4] * log(Cr * day) +
                                         A[5] * log(Cr * day) * log(NH4)) / (Nr * day) * O2 / (kO2 + O2));
    const double* B = p->denitrification;
    const double pd = or_mg_fraction(exp(B[0] + B[1] * log(Cr * day) + B[2] * pow(log(NO3), 2) +
                                         B[3] * pow(log(Cr * day), 2) + B[4] * pow(log(k * day), 2) +
                                         B[5] * log(O2) * log(k)) / (Cr * day) * O2 / (kO2 + O2));
    const double* Cc = p->anoxic;
    const double pa = or_mg_fraction(exp(Cc[0] + Cc[1] * log(Cr * day) + Cc[2] * pow(log(Cr * day), 2) +
                                         Cc[3] * log(k * day) + Cc[4] * log(O2) * log(k) +
                                         Cc[5] * pow(log(NO3), 2)) / (Cr * day));
    const double ps = 0.223 * pow(p->sedimentation_rate, 0.336);
    F[1] = (1 - pn) * Nr + 0.8 * pd * Cr;
    F[0] = pn * Nr - 0.8 * pd * Cr;
    F[2] = -(1 - pa * ps - pd) * O2 / (kO2 + O2) * Cr - 2 * pn * Nr;
}

/* update_biogeochemical_state!(model, sediment) (src/Sediments/update_state.jl:6-17): track the
 * bottom cells of `state` (tracked_fields.jl), take a full RK3 step of length dt (none for dt = 0;
 * timesteppers.jl:48-73, the first stage from the tendency cached by the previous step's
 * update_state!, computed afresh on the first step), then the coupled tendencies F[3][NN]
 * (tracer_coupling.jl) for the next water stage. */
static void or_mg_update(const or_model3d* m, const double* state, const double* drift, double dt, double* F) {
    const or_multig* g = m->multig;
    const int Nx = m->grid.Nx, Ny = m->grid.Ny, Nz = m->grid.Nz;
    const long NN = (long)Nx * Ny, N = NN * Nz;
    for (long col = 0; col < NN; col++) {
        double dep = 0.0;   /* sinking_flux: minus the advective flux through the bottom face */
        for (int s = 0; s < g->n_sinking; s++) {
            const int q = g->sinking_slot[s];
            dep -= drift[(long)q * (Nz + 1)] * state[(long)q * N + col];
        }
        double* S = g->state;
        double x[3] = {S[col], S[NN + col], S[2 * NN + col]};
        if (dt > 0.0) {
            double G0[3], G1[3], G2[3];
            if (S[3 * NN + col] == 0.0) {
                or_mg_tendency(&g->p, x[0], x[1], dep, G0);
                S[3 * NN + col] = 1.0;
            } else {
                for (int q = 0; q < 3; q++) G0[q] = g->gcache[q * NN + col];
            }
            for (int q = 0; q < 3; q++) x[q] += dt * RK_G[0] * G0[q];
            or_mg_tendency(&g->p, x[0], x[1], dep, G1);
            for (int q = 0; q < 3; q++) x[q] += dt * (RK_G[1] * G1[q] + RK_Z[1] * G0[q]);
            or_mg_tendency(&g->p, x[0], x[1], dep, G2);
            for (int q = 0; q < 3; q++) x[q] += dt * (RK_G[2] * G2[q] + RK_Z[2] * G1[q]);
            or_mg_tendency(&g->p, x[0], x[1], dep, G0);
            for (int q = 0; q < 3; q++) { g->gcache[q * NN + col] = G0[q]; S[q * NN + col] = x[q]; }
        }
        double f[3];
        or_mg_coupling(&g->p, x[0], x[1], state[(long)g->no3 * N + col], state[(long)g->nh4 * N + col],
                       state[(long)g->o2 * N + col], f);
        for (int q = 0; q < 3; q++) F[q * NN + col] = f[q];
    }
}

/* nsteps RK3 steps; or, with only_stage in 0..2, that one stage of one step, with the tendency
 * arrays supplied by the caller (Gx receives the stage's tendency, Gmx holds the previous stage's,
 * sedx the sediment's previous-stage burial) and no modifier applied to the entering state. */
static void step3d_impl(const or_model3d* m, double* state, const double* u, const double* v,
                        const double* w, double t, double dt, int nsteps, int nthreads, int only_stage,
                        double* Gx, double* Gmx, double* sedx) {
    const obgc_grid* g = &m->grid;
    int Nx = g->Nx, Ny = g->Ny, Nz = g->Nz, nt = m->n_tracers;
    long NN = (long)Nx * Ny, N = NN * Nz;
    double dx = g->Lx / Nx, dy = g->Ly / Ny, dz = g->Lz / Nz;
    int px = g->topology_x == OBGC_PERIODIC, py = g->topology_y == OBGC_PERIODIC;
    int flat_y = g->topology_y == OBGC_FLAT || Ny == 1;
    int flat_x = g->topology_x == OBGC_FLAT;
    const int ext = only_stage >= 0;
    double* G = ext ? Gx : calloc((size_t)nt * N, sizeof(double));
    double* Gm = ext ? Gmx : calloc((size_t)nt * N, sizeof(double));
    double* PAR = malloc(sizeof(double) * N);
    double* drift = calloc((size_t)nt * (Nz + 1), sizeof(double));
    int* has_drift = calloc(nt, sizeof(int));
    double* sed_Gm = ext ? sedx : calloc((size_t)NN, sizeof(double));
    int32_t req[32];
    int nreq = or_npd_required_tracers(&m->npd, req, 32);
    int is_bgc[32] = {0};
    for (int q = 0; q < nt; q++) {
        for (int r = 0; r < nreq; r++) if (m->names[q] == req[r]) is_bgc[q] = 1;
        if (m->names[q] >= 0 && m->advection) {
            or_npd_drift_profile(&m->npd, m->names[q], Nz, drift + (long)q * (Nz + 1), &has_drift[q]);
            if (has_drift[q]) {
                int nz = 0;
                for (int f = 0; f <= Nz; f++) nz |= drift[(long)q * (Nz + 1) + f] != 0.0;
                has_drift[q] = nz;
            }
        }
    }
    int32_t gn[OR_MAX_GROUPS], gslot[OR_MAX_GROUPS * OR_MAX_GROUP];
    double gfac[OR_MAX_GROUPS * OR_MAX_GROUP];
    const int ng = m->negatives == 1 ? or_conserved_groups(&m->npd, nt, m->names, gn, gslot, gfac) : 0;
    if (m->negatives && !ext) or_negatives3d(m, state, N, ng, gn, gslot, gfac, nthreads);
    /* the SimpleMultiG sediment's coupled tendencies of the entering state (full steps only) */
    double* mgF = (m->multig && !ext) ? calloc((size_t)3 * NN, sizeof(double)) : NULL;
    if (mgF) or_mg_update(m, state, drift, 0.0, mgF);
    const int st0 = ext ? only_stage : 0, st1 = ext ? only_stage + 1 : 3;
    for (int s = 0; s < nsteps; s++) {
        for (int st = st0; st < st1; st++) {
            double ts = t + RK_C[st] * dt;
            or_par3d(m, state, ts, PAR, nthreads);
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (long c = 0; c < N; c++) {
                int i = (int)(c % Nx), j = (int)((c / Nx) % Ny), k = (int)(c / NN);
                double vals[OBGC_NUM_NAMED] = {0};
                for (int q = 0; q < nt; q++) if (m->names[q] >= 0) vals[m->names[q]] = state[(long)q * N + c];
                for (int q = 0; q < nt; q++) {
                    /* a replicate (DIC2, Alk2, ...) evaluates the DIC / Alk functor
                     * (carbonate_system.jl:70-83); a forcing adds its rate at the stage time */
                    double tend = is_bgc[q] ? or_npd_tendency(&m->npd, m->names[q], vals, PAR[c])
                                : m->tendency_of[q] > 0 ? or_npd_tendency(&m->npd, m->tendency_of[q] - 1, vals, PAR[c])
                                : 0.0;
                    if (m->forcing[q] && ts >= m->forcing_t0[q] && ts < m->forcing_t1[q]) tend += m->forcing[q][c];
                    if (m->advection) {
                        const double* cq = state + (long)q * N;
                        double adv = 0.0;
                        if (!flat_x && u) {
                            const double* line = cq + (long)k * NN + (long)j * Nx;
                            int f0 = i, f1 = i + 1;
                            double U0 = (px || (f0 > 0 && f0 < Nx)) ? u[(long)k * NN + (long)j * Nx + (f0 % Nx)] : 0.0;
                            double U1 = (px || (f1 > 0 && f1 < Nx)) ? u[(long)k * NN + (long)j * Nx + (f1 % Nx)] : 0.0;
                            double F0 = U0 != 0.0 ? U0 * face_value(line, 1, Nx, px, f0, U0) : 0.0;
                            double F1 = U1 != 0.0 ? U1 * face_value(line, 1, Nx, px, f1, U1) : 0.0;
                            adv += (F1 - F0) / dx;
                        }
                        if (!flat_y && v) {
                            const double* line = cq + (long)k * NN + i;
                            int f0 = j, f1 = j + 1;
                            double V0 = (py || (f0 > 0 && f0 < Ny)) ? v[(long)k * NN + (long)(f0 % Ny) * Nx + i] : 0.0;
                            double V1 = (py || (f1 > 0 && f1 < Ny)) ? v[(long)k * NN + (long)(f1 % Ny) * Nx + i] : 0.0;
                            double F0 = V0 != 0.0 ? V0 * face_value(line, Nx, Ny, py, f0, V0) : 0.0;
                            double F1 = V1 != 0.0 ? V1 * face_value(line, Nx, Ny, py, f1, V1) : 0.0;
                            adv += (F1 - F0) / dy;
                        }
                        const double* zline = cq + (long)j * Nx + i;
                        if (w) {
                            double W0 = (k > 0) ? w[(long)k * NN + (long)j * Nx + i] : 0.0;
                            double W1 = (k + 1 < Nz) ? w[(long)(k + 1) * NN + (long)j * Nx + i] : 0.0;
                            double F0 = W0 != 0.0 ? W0 * face_value(zline, NN, Nz, 0, k, W0) : 0.0;
                            double F1 = W1 != 0.0 ? W1 * face_value(zline, NN, Nz, 0, k + 1, W1) : 0.0;
                            adv += (F1 - F0) / dz;
                        }
                        if (has_drift[q]) {
                            const double* wd = drift + (long)q * (Nz + 1);
                            double W0 = wd[k], W1 = wd[k + 1];
                            double F0 = W0 != 0.0 ? W0 * face_value(zline, NN, Nz, 0, k, W0) : 0.0;
                            double F1 = W1 != 0.0 ? W1 * face_value(zline, NN, Nz, 0, k + 1, W1) : 0.0;
                            adv += (F1 - F0) / dz;
                        }
                        tend -= adv;
                    }
                    if (m->kappa_h > 0.0 || m->kappa_z_faces) {
                        /* ScalarDiffusivity, explicit: -div(-kappa grad c) with no flux through walls */
                        const double* cq = state + (long)q * N;
                        const int fx = g->topology_x == OBGC_FLAT, fy = g->topology_y == OBGC_FLAT || Ny == 1;
                        double d = 0.0;
                        if (!fx && m->kappa_h > 0.0) {
                            const long row = (long)k * NN + (long)j * Nx;
                            const double cm = (px || i > 0) ? cq[row + (i + Nx - 1) % Nx] : cq[row + i];
                            const double cp = (px || i < Nx - 1) ? cq[row + (i + 1) % Nx] : cq[row + i];
                            d += m->kappa_h * (cp - 2 * cq[row + i] + cm) / (dx * dx);
                        }
                        if (!fy && m->kappa_h > 0.0) {
                            const long base = (long)k * NN + i;
                            const double cm = (py || j > 0) ? cq[base + (long)((j + Ny - 1) % Ny) * Nx] : cq[base + (long)j * Nx];
                            const double cp = (py || j < Ny - 1) ? cq[base + (long)((j + 1) % Ny) * Nx] : cq[base + (long)j * Nx];
                            d += m->kappa_h * (cp - 2 * cq[base + (long)j * Nx] + cm) / (dy * dy);
                        }
                        if (m->kappa_z_faces && !m->vertical_implicit) {
                            const double cc = cq[c];
                            const double up = k + 1 < Nz ? m->kappa_z_faces[k + 1] * (cq[c + NN] - cc) : 0.0;
                            const double dn = k > 0 ? m->kappa_z_faces[k] * (cc - cq[c - NN]) : 0.0;
                            d += (up - dn) / (dz * dz);
                        }
                        tend += d;
                    }
                    G[(long)q * N + c] = tend;
                }
            }
            /* FieldBoundaryConditions(top = GasExchange): the surface cell loses flux / dz
             * (gas_exchange.jl:26-39 evaluated on the stage's surface values) */
            for (int gq = 0; gq < OR_MAX_GAS; gq++) {
                const obgc_gas_exchange* ge = m->gas[gq];
                if (!ge) continue;
                int sT = -1, sS = -1;
                for (int q = 0; q < nt; q++) {
                    if (m->names[q] == OBGC_T) sT = q;
                    if (m->names[q] == OBGC_S) sS = q;
                }
                const int target = m->gas_target[gq];
                const int co2 = ge->gas == OBGC_GAS_CO2;
                const int sD = co2 ? m->gas_dic[gq] : -1, sA = co2 ? m->gas_alk[gq] : -1, sO = co2 ? -1 : target;
                if (sT < 0 || sS < 0 || target < 0 || (co2 && (sA < 0 || sD < 0))) continue;
#pragma omp parallel for num_threads(nthreads) schedule(static)
                for (long col = 0; col < NN; col++) {
                    const long c = (long)(Nz - 1) * NN + col;
                    const double F = or_gas_exchange_flux(ge, state[(long)sT * N + c], state[(long)sS * N + c],
                                                          sD >= 0 ? state[(long)sD * N + c] : 0.0,
                                                          sA >= 0 ? state[(long)sA * N + c] : 0.0,
                                                          sO >= 0 ? state[(long)sO * N + c] : 0.0, ge->wind_speed,
                                                          ge->air_concentration);
                    G[(long)target * N + c] -= F / dz;
                }
            }
            /* SimpleMultiG: the coupled tendencies enter the bottom cells (tracer_coupling.jl) */
            if (mgF) {
                const int slots[3] = {m->multig->no3, m->multig->nh4, m->multig->o2};
                for (long col = 0; col < NN; col++)
                    for (int q = 0; q < 3; q++) G[(long)slots[q] * N + col] += mgF[q * NN + col] / dz;
            }
            /* InstantRemineralisationSediment (instant_remineralisation.jl:96-120; tracer_coupling.jl,
             * tracked_fields.jl): the sinking fluxes through the bottom face deposit F, a fraction
             * e = a + b (F/(k+F))^2 is buried, the rest returns to the receiver's bottom cell */
            if (m->sed_receiver >= 0 && m->sed_storage) {
                const double gs = RK_G[st], zs = RK_Z[st];
                for (long col = 0; col < NN; col++) {
                    double dep = 0.0;
                    for (int q = 0; q < nt; q++) {
                        if (!((m->sed_sink_mask >> q) & 1u) || !has_drift[q]) continue;
                        const double W0 = drift[(long)q * (Nz + 1)];
                        const double* zline = state + (long)q * N + col;
                        const double F0 = W0 != 0.0 ? W0 * face_value(zline, NN, Nz, 0, 0, W0) : 0.0;
                        dep -= F0;
                    }
                    const double r = dep / (m->sed_k + dep);
                    const double e = m->sed_a + m->sed_b * (r * r);
                    G[(long)m->sed_receiver * N + col] += (1.0 - e) * dep / dz;
                    const double burial = e * dep;
                    m->sed_storage[col] += st == 0 ? dt * gs * burial : dt * (gs * burial + zs * sed_Gm[col]);
                    sed_Gm[col] = burial;
                }
            }
            double g = RK_G[st], z = RK_Z[st];
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (long x = 0; x < (long)nt * N; x++) {
                if (st == 0) state[x] += dt * g * G[x];
                else state[x] += dt * (g * G[x] + z * Gm[x]);
            }
            if (m->stage_rounding > 0.0) {
                const uint64_t stage_count = (uint64_t)s * 3u + (uint64_t)st;
#pragma omp parallel for num_threads(nthreads) schedule(static)
                for (long x = 0; x < (long)nt * N; x++) {
                    const uint64_t h = mix64((uint64_t)x * 0x9E3779B97F4A7C15ull ^ (stage_count << 40) ^ m->rounding_seed);
                    state[x] *= 1.0 + ((h >> 63) ? m->stage_rounding : -m->stage_rounding);
                }
            }
            /* VerticallyImplicitTimeDiscretization: (I - dt_s d/dz kappa d/dz) U = U* per column and
             * tracer with dt_s = (gamma + zeta) dt, walls at the bottom and top */
            if (m->kappa_z_faces && m->vertical_implicit) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
                for (long qc = 0; qc < (long)nt * NN; qc++) {
                    const long q = qc / NN, col = qc % NN;
                    double x[Nz], cp[Nz], dp[Nz];
                    for (int k = 0; k < Nz; k++) x[k] = state[q * N + (long)k * NN + col];
                    implicit_diffusion(Nz, dz, m->kappa_z_faces, (g + z) * dt, x, cp, dp);
                    for (int k = 0; k < Nz; k++) state[q * N + (long)k * NN + col] = x[k];
                }
            }
            if (m->negatives) or_negatives3d(m, state, N, ng, gn, gslot, gfac, nthreads);
            /* update_state!: the sediment tracks the new state and steps the stage's length */
            if (mgF) or_mg_update(m, state, drift, (g + z) * dt, mgF);
            double* tmp = G; G = Gm; Gm = tmp;
        }
        t += dt;
    }
    if (!ext) { free(G); free(Gm); free(sed_Gm); }
    free(mgF);
    free(PAR); free(drift); free(has_drift);
}

void or_step3d(const or_model3d* m, double* state, const double* u, const double* v,
               const double* w, double t, double dt, int nsteps, int nthreads) {
    step3d_impl(m, state, u, v, w, t, dt, nsteps, nthreads, -1, NULL, NULL, NULL);
}

void or_stage3d(const or_model3d* m, double* state, const double* u, const double* v, const double* w,
                double t, double dt, int stage, double* G, double* Gm, double* sed_Gm, int nthreads) {
    if (stage < 0 || stage > 2) return;
    step3d_impl(m, state, u, v, w, t, dt, 1, nthreads, stage, G, Gm, sed_Gm);
}

/* ------------------------------------------------------------------ negative tracers -- */
static int slot_in(int nt, const int32_t* names, int name) {
    for (int q = 0; q < nt; q++) if (names[q] == name) return q;
    return -1;
}

static void group_add(int nt, const int32_t* names, int g, int name, double f, int32_t* gn, int32_t* gslot, double* gfac) {
    int q = slot_in(nt, names, name);
    if (q < 0 || gn[g] >= OR_MAX_GROUP) return;
    gslot[g * OR_MAX_GROUP + gn[g]] = q;
    gfac[g * OR_MAX_GROUP + gn[g]] = f;
    gn[g]++;
}

int or_conserved_groups(const obgc_npd_params* p, int nt, const int32_t* names, int32_t* gn, int32_t* gslot,
                        double* gfac) {
    gn[0] = gn[1] = 0;
    /* nitrogen: P, Z, nutrients, detritus (coupling_utils.jl:1-21) */
    group_add(nt, names, 0, OBGC_P, 1.0, gn, gslot, gfac);
    group_add(nt, names, 0, OBGC_Z, 1.0, gn, gslot, gfac);
    if (p->nutrients == OBGC_NUT_NUTRIENT) group_add(nt, names, 0, OBGC_N, 1.0, gn, gslot, gfac);
    else { group_add(nt, names, 0, OBGC_NO3, 1.0, gn, gslot, gfac); group_add(nt, names, 0, OBGC_NH4, 1.0, gn, gslot, gfac); }
    if (p->detritus == OBGC_DET_VARIABLE_REDFIELD) {
        group_add(nt, names, 0, OBGC_SPON, 1.0, gn, gslot, gfac); group_add(nt, names, 0, OBGC_BPON, 1.0, gn, gslot, gfac);
        group_add(nt, names, 0, OBGC_DON, 1.0, gn, gslot, gfac);
    } else if (p->detritus == OBGC_DET_TWO_PARTICLE) {
        group_add(nt, names, 0, OBGC_SPOM, 1.0, gn, gslot, gfac); group_add(nt, names, 0, OBGC_BPOM, 1.0, gn, gslot, gfac);
        group_add(nt, names, 0, OBGC_DOM, 1.0, gn, gslot, gfac);
    } else if (p->detritus == OBGC_DET_SINGLE) {
        group_add(nt, names, 0, OBGC_D, 1.0, gn, gslot, gfac);
    }
    if (!p->carbonate_system) return 1;
    /* carbon: P, Z, DIC, detritus carbon with ((1 + rho) R, R, 1, ...) (coupling_utils.jl:23-52) */
    const double R = p->redfield_ratio, rho = p->carbon_calcite_ratio;
    group_add(nt, names, 1, OBGC_P, (1 + rho) * R, gn, gslot, gfac);
    group_add(nt, names, 1, OBGC_Z, R, gn, gslot, gfac);
    group_add(nt, names, 1, OBGC_DIC, 1.0, gn, gslot, gfac);
    if (p->detritus == OBGC_DET_VARIABLE_REDFIELD) {
        group_add(nt, names, 1, OBGC_SPOC, 1.0, gn, gslot, gfac); group_add(nt, names, 1, OBGC_BPOC, 1.0, gn, gslot, gfac);
        group_add(nt, names, 1, OBGC_DOC, 1.0, gn, gslot, gfac);
    } else if (p->detritus == OBGC_DET_TWO_PARTICLE) {
        group_add(nt, names, 1, OBGC_SPOM, R, gn, gslot, gfac); group_add(nt, names, 1, OBGC_BPOM, R, gn, gslot, gfac);
        group_add(nt, names, 1, OBGC_DOM, R, gn, gslot, gfac);
    } else if (p->detritus == OBGC_DET_SINGLE) {
        group_add(nt, names, 1, OBGC_D, R, gn, gslot, gfac);
    }
    return 2;
}

void or_scale_cell(double* v, long stride, int ng, const int32_t* gn, const int32_t* gslot, const double* gfac,
                   double fill) {
    for (int g = 0; g < ng; g++) {
        double t = 0.0, p = 0.0;
        for (int m = 0; m < gn[g]; m++) {
            double x = v[(long)gslot[g * OR_MAX_GROUP + m] * stride] * gfac[g * OR_MAX_GROUP + m];
            t += x;
            if (v[(long)gslot[g * OR_MAX_GROUP + m] * stride] > 0) p += x;
        }
        t = t < 0 ? fill : t;
        for (int m = 0; m < gn[g]; m++) {
            double* x = v + (long)gslot[g * OR_MAX_GROUP + m] * stride;
            *x = (!isfinite(*x) || *x > 0) ? *x * t / p : 0.0;
        }
    }
}

/* ------------------------------------------------------------------ columns ---------- */
/* Thomas solve of (I - dts * d/dz kappa d/dz) x = rhs on a column with zero-flux walls. */
static void implicit_diffusion(int Nz, double dz, const double* kf, double dts, double* x, double* cp, double* dp) {
    double r = dts / (dz * dz);
    for (int k = 0; k < Nz; k++) {
        double lo = k > 0 ? -r * kf[k] : 0.0;
        double up = k < Nz - 1 ? -r * kf[k + 1] : 0.0;
        double di = 1 - lo - up;
        if (k == 0) { cp[0] = up / di; dp[0] = x[0] / di; }
        else {
            double den = di - lo * cp[k - 1];
            cp[k] = up / den;
            dp[k] = (x[k] - lo * dp[k - 1]) / den;
        }
    }
    x[Nz - 1] = dp[Nz - 1];
    for (int k = Nz - 2; k >= 0; k--) x[k] = dp[k] - cp[k] * x[k + 1];
}

void or_columns_run(const obgc_npd_params* p0, const obgc_twoband_params* lp, int n_cols,
                    const or_column* cols, const int64_t* so, const int64_t* ko,
                    int nt, const int32_t* names, double* state, const double* kappa,
                    double t0, double dt_all, int nsteps_all, int negatives, double fill, int nthreads,
                    const obgc_gas_exchange* gas) {
    (void)t0;
    int32_t gn[OR_MAX_GROUPS], gslot[OR_MAX_GROUPS * OR_MAX_GROUP];
    double gfac[OR_MAX_GROUPS * OR_MAX_GROUP];
    const int ng = negatives == 1 ? or_conserved_groups(p0, nt, names, gn, gslot, gfac) : 0;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
    for (int c = 0; c < n_cols; c++) {
        obgc_npd_params p = *p0;
        if (cols[c].mu0 > 0) p.phytoplankton_maximum_growth_rate = cols[c].mu0;
        int Nz = cols[c].Nz;
        double dz = cols[c].dz;
        double dt = cols[c].dt > 0 ? cols[c].dt : dt_all;
        int nsteps = cols[c].nsteps > 0 ? cols[c].nsteps : nsteps_all;
        int sAlk = -1, sDIC = -1;
        for (int q = 0; q < nt; q++) {
            if (names[q] == OBGC_ALK) sAlk = q;
            if (names[q] == OBGC_DIC) sDIC = q;
        }
        double* U = state + so[c];
        const double* kf = kappa + ko[c];
        double* G = calloc((size_t)nt * Nz, sizeof(double));
        double* Gm = calloc((size_t)nt * Nz, sizeof(double));
        double* PAR = malloc(sizeof(double) * Nz);
        double* Pcol = malloc(sizeof(double) * Nz);
        double* zc = malloc(sizeof(double) * (Nz + 1));
        double* zf = malloc(sizeof(double) * (Nz + 1));
        double* wd = malloc(sizeof(double) * (size_t)nt * (Nz + 1));
        int* hd = calloc(nt, sizeof(int));
        double* cp = malloc(sizeof(double) * Nz);
        double* dp = malloc(sizeof(double) * Nz);
        for (int k = 0; k <= Nz; k++) zf[k] = -Nz * dz + k * dz;
        for (int k = 0; k < Nz; k++) zc[k] = -Nz * dz + (k + 0.5) * dz;
        int sP = -1;
        for (int q = 0; q < nt; q++) {
            if (names[q] == OBGC_P) sP = q;
            or_npd_drift_profile(&p, names[q], Nz, wd + (long)q * (Nz + 1), &hd[q]);
        }
        int32_t req[32];
        int nreq = or_npd_required_tracers(&p, req, 32);
        for (int k = 0; k < Nz && ng; k++) or_scale_cell(U + k, Nz, ng, gn, gslot, gfac, fill);
        for (int s = 0; s < nsteps; s++) {
            if (s == cols[c].pulse_step && sAlk >= 0 && cols[c].pulse_k >= 0 && cols[c].pulse_k < Nz)
                U[(long)sAlk * Nz + cols[c].pulse_k] += cols[c].pulse_amount;
            for (int st = 0; st < 3; st++) {
                for (int k = 0; k < Nz; k++) Pcol[k] = U[(long)sP * Nz + k];
                or_twoband_column(lp, Nz, zc, zf, Pcol, cols[c].surface_PAR, PAR);
                for (int k = 0; k < Nz; k++) {
                    double vals[OBGC_NUM_NAMED] = {0};
                    for (int q = 0; q < nt; q++) vals[names[q]] = U[(long)q * Nz + k];
                    for (int q = 0; q < nt; q++) {
                        int bgc = 0;
                        for (int r = 0; r < nreq; r++) bgc |= req[r] == names[q];
                        double tend = bgc ? or_npd_tendency(&p, names[q], vals, PAR[k]) : 0.0;
                        if (hd[q]) {
                            const double* w = wd + (long)q * (Nz + 1);
                            const double* line = U + (long)q * Nz;
                            double W0 = w[k], W1 = w[k + 1];
                            double F0 = W0 != 0.0 ? W0 * face_value(line, 1, Nz, 0, k, W0) : 0.0;
                            double F1 = W1 != 0.0 ? W1 * face_value(line, 1, Nz, 0, k + 1, W1) : 0.0;
                            tend -= (F1 - F0) / dz;
                        }
                        G[(long)q * Nz + k] = tend;
                    }
                }
                /* FieldBoundaryConditions(top = CarbonDioxideGasExchangeBoundaryCondition()) on DIC
                 * (examples/column.jl:54-64): the surface cell loses the stage's flux / dz */
                if (gas && sDIC >= 0 && sAlk >= 0) {
                    const long top = Nz - 1;
                    const double F = or_gas_exchange_flux(gas, cols[c].temperature, cols[c].salinity,
                                                          U[(long)sDIC * Nz + top], U[(long)sAlk * Nz + top], 0.0,
                                                          gas->wind_speed, gas->air_concentration);
                    G[(long)sDIC * Nz + top] -= F / dz;
                }
                double g = RK_G[st], z = RK_Z[st];
                for (long x = 0; x < (long)nt * Nz; x++)
                    U[x] += st == 0 ? dt * g * G[x] : dt * (g * G[x] + z * Gm[x]);
                for (int q = 0; q < nt; q++) implicit_diffusion(Nz, dz, kf, (g + z) * dt, U + (long)q * Nz, cp, dp);
                for (int k = 0; k < Nz && ng; k++) or_scale_cell(U + k, Nz, ng, gn, gslot, gfac, fill);
                double* tmp = G; G = Gm; Gm = tmp;
            }
        }
        free(G); free(Gm); free(PAR); free(Pcol); free(zc); free(zf); free(wd); free(hd); free(cp); free(dp);
    }
}

/* ------------------------------------------------------------------ negatives ---------- */
void or_scale_negatives(int64_t n, int ntr, double* const* fields, const double* sf, double fill) {
    for (int64_t c = 0; c < n; c++) {
        double t = 0.0, p = 0.0;
        for (int q = 0; q < ntr; q++) {
            double v = fields[q][c];
            t += v * sf[q];
            if (v > 0) p += v * sf[q];
        }
        t = t < 0 ? fill : t;
        for (int q = 0; q < ntr; q++) {
            double v = fields[q][c];
            fields[q][c] = (!isfinite(v) || v > 0) ? v * t / p : 0.0;
        }
    }
}

/* ------------------------------------------------------------------ PISCES 3-D ---------- */
void or_pisces_update_state3d(const or_pisces3d* m, const double* state, double t, double* par4, double* xy2,
                              double* omega, int nthreads) {
    const obgc_grid* g = &m->grid;
    const int Nx = g->Nx, Ny = g->Ny, Nz = g->Nz;
    const long NN = (long)Nx * Ny, N = NN * Nz;
    const double dz = g->Lz / Nz;
    const double PAR0 = m->surface_kind == OBGC_SURFACE_PAR_DEFAULT ? or_default_surface_PAR(t) : m->surface_value;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 8)
    for (long col = 0; col < NN; col++) {
        double zc[1024], zf[1025], chl[1024], band[1024], tot[1024];
        for (int k = 0; k <= Nz; k++) { zc[k] = -g->Lz + (k + 0.5) * dz; zf[k] = -g->Lz + k * dz; }
        for (int k = 0; k < Nz; k++) {
            chl[k] = state[(long)OBGC_PIS_PCHL * N + k * NN + col] + state[(long)OBGC_PIS_DCHL * N + k * NN + col];
            tot[k] = 0.0;
        }
        /* update_MultiBandPhotosyntheticallyActiveRadiation! (src/Light/multi_band.jl:147-185) */
        for (int b = 0; b < m->nbands; b++) {
            or_multiband_column(Nz, zc, m->kw[b], m->e[b], m->chi[b], chl, PAR0 * m->division[b], band);
            for (int k = 0; k < Nz; k++) {
                if (b < 3) par4[(long)(b + 1) * N + k * NN + col] = band[k];
                tot[k] += band[k];
            }
        }
        for (int k = 0; k < Nz; k++) par4[k * NN + col] = tot[k];
        /* compute_euphotic_depth! with the surface value of the total field */
        double zce[1025];
        for (int k = 0; k < Nz; k++) zce[k] = zc[k];
        zce[Nz] = -g->Lz - 0.5 * dz;   /* a column that never crosses the cutoff: the centre below the bottom */
        xy2[col] = or_euphotic_depth_column(Nz, zce, tot, 2 * PAR0 - tot[Nz - 1], 1e-3);
        /* compute_mean_mixed_layer_light! (mean_mixed_layer_properties.jl:105-106) */
        xy2[NN + col] = or_mixed_layer_mean(Nz, zf, tot, m->mixed_layer_depth);
    }
    /* compute_calcite_saturation! (compute_calcite_saturation.jl:23-36) */
    obgc_carbon_options o = m->carbon;
    o.output = OBGC_OUT_OMEGA_CALCITE;
    o.ph_given = 0;
    o.has_pressure = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (long c = 0; c < N; c++) {
        const int k = (int)(c / NN);
        const double z = -g->Lz + (k + 0.5) * dz;
        const double P = fabs(z) * 9.80665 * 1026 / 100000;
        double out = 0;
        or_carbon_chemistry(&o, state[(long)OBGC_PIS_DIC * N + c], state[(long)OBGC_PIS_ALK * N + c],
                            state[(long)OBGC_PIS_T * N + c], state[(long)OBGC_PIS_S * N + c], state[(long)OBGC_PIS_SI * N + c],
                            0.0, P, 0.0, &out, NULL);
        omega[c] = out;
    }
}

static void pisces_negatives(const or_pisces3d* m, double* state, long N, int nthreads) {
    if (m->negatives != 1) return;
    int32_t gn[OR_MAX_GROUPS], gslot[OR_MAX_GROUPS * OR_MAX_GROUP];
    double gfac[OR_MAX_GROUPS * OR_MAX_GROUP];
    const int ng = or_pisces_conserved_groups(&m->p, gn, gslot, gfac);
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (long c = 0; c < N; c++) or_scale_cell(state + c, N, ng, gn, gslot, gfac, m->invalid_fill_value);
}

/* The work buffers of a PISCES stage and the sinking speeds at the faces (POC at a constant speed,
 * GOC with DepthDependantSinkingSpeed evaluated at construction, euphotic depth 0), built as
 * setup_velocity_fields does. */
typedef struct {
    double *par4, *xy2, *omega, *wpoc, *wgoc, *zc;
} pisces_work;

static void pisces_work_init(const or_pisces3d* m, pisces_work* w) {
    const obgc_grid* g = &m->grid;
    const int Nz = g->Nz;
    const long NN = (long)g->Nx * g->Ny, N = NN * Nz;
    const double dz = g->Lz / Nz;
    w->par4 = malloc(sizeof(double) * 4 * N);
    w->xy2 = malloc(sizeof(double) * 2 * NN);
    w->omega = malloc(sizeof(double) * N);
    w->wpoc = malloc(sizeof(double) * (Nz + 1));
    w->wgoc = malloc(sizeof(double) * (Nz + 1));
    w->zc = malloc(sizeof(double) * (Nz + 1));
    for (int k = 0; k <= Nz; k++) w->zc[k] = -g->Lz + (k + 0.5) * dz;
    for (int f = 0; f <= Nz; f++)
        w->wpoc[f] = f < Nz ? -m->p.poc_sinking_speed * (m->p.open_bottom ? 1.0 : 1 - exp((double)(-f) / 2)) : 0.0;
    or_pisces_goc_speed(&m->p, Nz, w->zc, m->mixed_layer_depth, 0.0, w->wgoc);
}

static void pisces_work_free(pisces_work* w) {
    free(w->par4); free(w->xy2); free(w->omega); free(w->wpoc); free(w->wgoc); free(w->zc);
}

/* One RK3 stage st of the step that starts at t: update_state!, every tendency into G, the update
 * with the previous stage's Gm, then the negative-tracer modifier. */
static void pisces_stage(const or_pisces3d* m, double* state, const double* u, const double* v, double t, double dt,
                         int st, double* G, const double* Gm, pisces_work* w, int nthreads) {
    const obgc_grid* g = &m->grid;
    const int Nx = g->Nx, Ny = g->Ny, Nz = g->Nz, nt = OBGC_PIS_NUM;
    const long NN = (long)Nx * Ny, N = NN * Nz;
    const double dx = g->Lx / Nx, dy = g->Ly / Ny, dz = g->Lz / Nz;
    const int px = g->topology_x == OBGC_PERIODIC, py = g->topology_y == OBGC_PERIODIC;
    const int flat_x = g->topology_x == OBGC_FLAT || !m->advection, flat_y = g->topology_y == OBGC_FLAT || Ny == 1 || !m->advection;
    double *par4 = w->par4, *xy2 = w->xy2, *omega = w->omega, *wpoc = w->wpoc, *wgoc = w->wgoc, *zc = w->zc;
    const double ts = t + RK_C[st] * dt;
    or_pisces_update_state3d(m, state, ts, par4, xy2, omega, nthreads);
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (long c = 0; c < N; c++) {
        const int i = (int)(c % Nx), j = (int)((c / Nx) % Ny), k = (int)(c / NN);
        const long col = (long)j * Nx + i;
        double vals[OBGC_PIS_NUM], aux[OBGC_PAUX_NUM], Gb[OBGC_PIS_NUM_BGC];
        for (int q = 0; q < nt; q++) vals[q] = state[(long)q * N + c];
        aux[OBGC_PAUX_ZMXL] = m->mixed_layer_depth;
        aux[OBGC_PAUX_ZEU] = xy2[col];
        aux[OBGC_PAUX_SICLIM] = m->p.silicate_climatology;
        aux[OBGC_PAUX_OMEGA] = omega[c];
        aux[OBGC_PAUX_KAPPA] = m->mean_kappa;
        aux[OBGC_PAUX_MLPAR] = xy2[NN + col];
        aux[OBGC_PAUX_WPOC] = 0.5 * (wpoc[k] + wpoc[k + 1]);
        aux[OBGC_PAUX_WGOC] = 0.5 * (wgoc[k] + wgoc[k + 1]);
        aux[OBGC_PAUX_PAR] = par4[c];
        aux[OBGC_PAUX_PAR1] = par4[N + c];
        aux[OBGC_PAUX_PAR2] = par4[2 * N + c];
        aux[OBGC_PAUX_PAR3] = par4[3 * N + c];
        or_pisces_tendencies(&m->p, vals, aux, zc[k], ts, Gb);
        for (int q = 0; q < nt; q++) {
            double tend = q < OBGC_PIS_NUM_BGC ? Gb[q] : 0.0;
            const double* cq = state + (long)q * N;
            double adv = 0.0;
            if (!flat_x && u) {
                const double* line = cq + (long)k * NN + (long)j * Nx;
                int f0 = i, f1 = i + 1;
                double U0 = (px || (f0 > 0 && f0 < Nx)) ? u[(long)k * NN + (long)j * Nx + (f0 % Nx)] : 0.0;
                double U1 = (px || (f1 > 0 && f1 < Nx)) ? u[(long)k * NN + (long)j * Nx + (f1 % Nx)] : 0.0;
                double F0 = U0 != 0.0 ? U0 * face_value(line, 1, Nx, px, f0, U0) : 0.0;
                double F1 = U1 != 0.0 ? U1 * face_value(line, 1, Nx, px, f1, U1) : 0.0;
                adv += (F1 - F0) / dx;
            }
            if (!flat_y && v) {
                const double* line = cq + (long)k * NN + i;
                int f0 = j, f1 = j + 1;
                double V0 = (py || (f0 > 0 && f0 < Ny)) ? v[(long)k * NN + (long)(f0 % Ny) * Nx + i] : 0.0;
                double V1 = (py || (f1 > 0 && f1 < Ny)) ? v[(long)k * NN + (long)(f1 % Ny) * Nx + i] : 0.0;
                double F0 = V0 != 0.0 ? V0 * face_value(line, Nx, Ny, py, f0, V0) : 0.0;
                double F1 = V1 != 0.0 ? V1 * face_value(line, Nx, Ny, py, f1, V1) : 0.0;
                adv += (F1 - F0) / dy;
            }
            /* biogeochemical_drift_velocity (two_size_class.jl:100-107) */
            const double* wd = NULL;
            if (m->advection && (q == OBGC_PIS_POC || q == OBGC_PIS_SFE)) wd = wpoc;
            if (m->advection && (q == OBGC_PIS_GOC || q == OBGC_PIS_BFE || q == OBGC_PIS_PSI || q == OBGC_PIS_CACO3)) wd = wgoc;
            if (wd) {
                const double* zline = cq + (long)j * Nx + i;
                double W0 = wd[k], W1 = wd[k + 1];
                double F0 = W0 != 0.0 ? W0 * face_value(zline, NN, Nz, 0, k, W0) : 0.0;
                double F1 = W1 != 0.0 ? W1 * face_value(zline, NN, Nz, 0, k + 1, W1) : 0.0;
                adv += (F1 - F0) / dz;
            }
            G[(long)q * N + c] = tend - adv;
        }
    }
    const double gg = RK_G[st], z = RK_Z[st];
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (long x = 0; x < (long)nt * N; x++) {
        if (st == 0) state[x] += dt * gg * G[x];
        else state[x] += dt * (gg * G[x] + z * Gm[x]);
    }
    pisces_negatives(m, state, N, nthreads);
}

void or_pisces_step3d(const or_pisces3d* m, double* state, const double* u, const double* v, double t, double dt,
                      int nsteps, int nthreads) {
    const long N = (long)m->grid.Nx * m->grid.Ny * m->grid.Nz;
    double* G = calloc((size_t)OBGC_PIS_NUM * N, sizeof(double));
    double* Gm = calloc((size_t)OBGC_PIS_NUM * N, sizeof(double));
    pisces_work w;
    pisces_work_init(m, &w);
    pisces_negatives(m, state, N, nthreads);
    for (int s = 0; s < nsteps; s++) {
        for (int st = 0; st < 3; st++) {
            pisces_stage(m, state, u, v, t, dt, st, G, Gm, &w, nthreads);
            double* tmp = G; G = Gm; Gm = tmp;
        }
        t += dt;
    }
    free(G); free(Gm);
    pisces_work_free(&w);
}

void or_pisces_stage3d(const or_pisces3d* m, double* state, const double* u, const double* v, double t, double dt,
                       int stage, double* G, const double* Gm, int start, int nthreads) {
    pisces_work w;
    pisces_work_init(m, &w);
    if (start) pisces_negatives(m, state, (long)m->grid.Nx * m->grid.Ny * m->grid.Nz, nthreads);
    pisces_stage(m, state, u, v, t, dt, stage, G, Gm, &w, nthreads);
    pisces_work_free(&w);
}

