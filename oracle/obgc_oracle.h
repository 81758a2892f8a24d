/*
 * obgc_oracle.h — TEST INFRASTRUCTURE, NOT THE PRODUCT.
 *
 * A CPU, FP64 restatement of OceanBioME.jl's tracer-tendency path (NutrientsPlanktonDetritus
 * functors, TwoBand/MultiBand light, CarbonChemistry + root solvers, BoxModel RK3) plus a
 * restatement of the third-party Oceananigans pieces the path runs inside (WENO5 tracer
 * advection, RK3 substeps, vertically implicit diffusion).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it, and only as the oracle the GPU results are compared with.  It shares nothing with
 * the CUDA product but the parameter structs of include/obgc.h (the interface).
 *
 * Parity pins: the reference's own known-answer tests (test/test_light.jl, test/test_solvers.jl,
 * test/test_gasexchange_carbon_chem.jl, test/test_NutrientsPlanktonDetritus.jl) and the
 * CarbonChemistry doctest digits (src/Models/CarbonChemistry/carbon_chemistry.jl:55-62).  WENO5
 * and RK3 come from Oceananigans, which is absent here: those are restated from the published
 * methods and are "parity unpinned" against the reference.
 */
#ifndef OBGC_ORACLE_H
#define OBGC_ORACLE_H
#include <stdint.h>
#include "../include/obgc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- NutrientsPlanktonDetritus ---- */
int or_npd_preset(int preset, obgc_npd_params* out);
int or_npd_required_tracers(const obgc_npd_params* p, int32_t* names, int cap);
double or_npd_tendency(const obgc_npd_params* p, int name, const double* v, double PAR);
void or_npd_drift_profile(const obgc_npd_params* p, int name, int Nz, double* w, int* drifts);

/* ---- light ---- */
void or_twoband_column(const obgc_twoband_params* lp, int Nz, const double* zc, const double* zf,
                       const double* P, double PAR0, double* PAR);
void or_multiband_column(int Nz, const double* zc, double kw, double e, double chi,
                         const double* Chl, double surface, double* PAR);
double or_euphotic_depth_column(int Nz, const double* zc, const double* PAR, double PAR_top_halo,
                                double cutoff);
void or_multiband_coefficients(int nbands, const double* band_edges, int nbase,
                               const double* lambda, const double* kw, const double* e,
                               const double* chi, double* okw, double* oe, double* ochi);
double or_default_surface_PAR(double t);

/* ---- carbon chemistry ---- */
enum { OR_K0 = 0, OR_K1, OR_K2, OR_KB, OR_KW, OR_KS, OR_KF, OR_KP1, OR_KP2, OR_KP3, OR_KSI,
       OR_KSP_CALCITE, OR_KSP_ARAGONITE, OR_NUM_K };
double or_equilibrium_constant(int which, double Tk, double S, int has_P, double P);
double or_pressure_correction(int which, double Tk, double P);
double or_first_virial(double Tk);
double or_cross_virial(double Tk);
double or_density_eos80(double T, double S, double Pbar);
double or_density_teos10_polynomial(double T, double S, double Pbar);
double or_density(const obgc_carbon_options* o, double T, double S, double Pbar);
int or_carbon_default_options(obgc_carbon_options* o);
int or_carbon_chemistry(const obgc_carbon_options* o, double DIC, double Alk, double T, double S,
                        double silicate, double phosphate, double P, double pH, double* out,
                        int* iters);
void or_carbon_chemistry_batch(const obgc_carbon_options* o, int64_t n, const double* DIC,
                               const double* Alk, const double* T, const double* S,
                               const double* Si, const double* PO4, const double* P,
                               const double* pH, double* out, int nthreads);

/* ---- root solvers (src/Utils/solvers.jl) on the test functions of test/test_solvers.jl ---- */
enum { OR_SOLVER_NEWTON = 0, OR_SOLVER_NEWTON_SAFE, OR_SOLVER_BISECTION, OR_SOLVER_DAMPED };
double or_solve_test_function(int solver, int fid, double x0, double x1, double damping,
                              double pa, double pb);

/* ---- BoxModel ---- */
void or_box_run_drivers(const obgc_npd_params* p, double* v, const double* PAR_stages, double PAR_const, double dt,
                        int nsteps, int np, const int32_t* pnames, const double* const* presc, int nf,
                        const int32_t* fnames, const double* const* frc);
void or_box_run(const obgc_npd_params* p, double* v, const double* PAR_stages, double PAR_const,
                double t0, double dt, int nsteps);

/* ---- 3-D fused model: WENO5 + drift + BGC + TwoBand light + RK3 ---- */
#define OR_MAX_GAS 4
/* SimpleMultiGSediment, nitrogen-only form (src/Models/Sediments/simple_multi_G.jl:15-430) coupled
 * as BiogeochemicalSediment (src/Sediments/): after every water RK3 stage the bottom cells are
 * tracked, the fields take a full RK3 step of the stage's length (first stage from the tendency
 * cached at the end of the previous step), and the coupled tendencies enter the next stage. */
typedef struct or_multig {
    obgc_multig_params p;        /* sedimentation_rate resolved (> 0)                          */
    int32_t n_sinking;
    int32_t sinking_slot[4];
    int32_t no3, nh4, o2;        /* slots of the coupled tracers                                */
    double* state;               /* [4][Ny*Nx]: Ns, Nf, Nr, started                              */
    double* gcache;              /* [3][Ny*Nx]: the fields' tendency at the end of the last step */
} or_multig;

typedef struct or_model3d {
    obgc_npd_params npd;
    obgc_twoband_params light;
    int32_t surface_kind;        /* enum obgc_surface_par (FIELD not supported here) */
    int32_t advection;           /* enum obgc_advection */
    double surface_value;
    obgc_grid grid;              /* strides ignored: arrays are dense [Nz][Ny][Nx]   */
    int32_t n_tracers;           /* number of advected tracers                         */
    int32_t names[32];           /* enum obgc_tracer per tracer, or -1 for passive     */
    int32_t negatives;           /* 0 none, 1 ScaleNegativeTracers, 2 ZeroNegativeTracers */
    int32_t zero_exclude_mask;   /* ZeroNegativeTracers: bit q set = tracer slot q excluded */
    double invalid_fill_value;   /* ScaleNegativeTracers(...; invalid_fill_value)      */
    const obgc_gas_exchange* gas[OR_MAX_GAS]; /* top boundary conditions (NULL: none), with
                                      * constant wind speed and air concentration: gas[q] takes
                                      * the flux out of slot gas_target[q]; CO2 reads the water's
                                      * DIC / Alk from slots gas_dic[q] / gas_alk[q], O2 the target */
    int32_t gas_target[OR_MAX_GAS], gas_dic[OR_MAX_GAS], gas_alk[OR_MAX_GAS];
    double kappa_h;                  /* ScalarDiffusivity: horizontal diffusivity (m2/s)         */
    const double* kappa_z_faces;     /* vertical diffusivity at the Nz + 1 faces, or NULL; the
                                      * bottom and top faces are walls (no flux)                  */
    int32_t vertical_implicit;       /* VerticallyImplicitTimeDiscretization: the vertical part is
                                      * solved implicitly after each stage's explicit update      */
    int32_t sed_receiver;            /* InstantRemineralisation: receiver tracer slot, or -1    */
    uint32_t sed_sink_mask;          /* sinking tracer slots                                     */
    double sed_a, sed_b, sed_k;      /* burial efficiency constants and half saturation          */
    double* sed_storage;             /* [Ny*Nx] storage, stepped with the tracers' RK3           */
    int32_t tendency_of[32];         /* passive slots (names -1): enum obgc_tracer + 1 whose BGC
                                      * tendency the slot takes (CarbonateSystem replicates), 0 none */
    const double* forcing[32];       /* per slot: a source rate [Nz*Ny*Nx] (per second) or NULL,  */
    double forcing_t0[32], forcing_t1[32]; /* added at stage times t0 <= t < t1              */
    double stage_rounding;           /* conditioning probe, 0 = off: after every stage each state
                                      * value is multiplied by (1 +/- stage_rounding), the sign
                                      * drawn from a hash of (value index, stage count, seed): a
                                      * model of one rounding of that relative size per stored value */
    uint64_t rounding_seed;
    const or_multig* multig;         /* SimpleMultiG sediment, or NULL                              */
} or_model3d;
/* state: [n_tracers][Nz*Ny*Nx]; u, v, w: [Nz*Ny*Nx] or NULL. */
void or_step3d(const or_model3d* m, double* state, const double* u, const double* v,
               const double* w, double t, double dt, int nsteps, int nthreads);
void or_par3d(const or_model3d* m, const double* state, double t, double* PAR, int nthreads);
/* One RK3 stage (0, 1, 2) of the step starting at t: G[n_tracers*N] receives the stage's
 * tendency, Gm holds the previous stage's (unused by stage 0), sed_Gm[Ny*Nx] the sediment's
 * previous-stage burial (or NULL without a sediment); the caller swaps G and Gm between stages.
 * No modifier is applied to the entering state (or_step3d applies it once before its first stage).
 * The stage-level form lets a domain split into y slabs exchange halo rows between stages. */
void or_stage3d(const or_model3d* m, double* state, const double* u, const double* v, const double* w,
                double t, double dt, int stage, double* G, double* Gm, double* sed_Gm, int nthreads);

/* ---- batched uneven columns with vertically implicit diffusion ---- */
typedef struct or_column {
    int32_t Nz;
    int32_t nsteps;              /* steps of this column (<= 0: the call's nsteps)        */
    double dz;
    double surface_PAR;          /* constant surface PAR (W/m2)                          */
    double mu0;                  /* phytoplankton_maximum_growth_rate override           */
    double dt;                   /* step of this column (<= 0: the call's dt)            */
    int32_t pulse_step;          /* step at whose start pulse_amount is added to Alk (-1) */
    int32_t pulse_k;
    double pulse_amount;
    double temperature, salinity; /* surface T and S of the CO2 gas exchange                   */
} or_column;
/* state: per column [n_tracers][Nz] (offsets given); kappa: per column Nz+1 face values.
 * negatives: 0 none, 1 ScaleNegativeTracers over conserved_tracers(bgc) (applied to the initial
 * state and after every RK3 stage, as Oceananigans' update_state! does). */
void or_columns_run(const obgc_npd_params* p, const obgc_twoband_params* lp, int n_cols,
                    const or_column* cols, const int64_t* state_offsets,
                    const int64_t* kappa_offsets, int n_tracers, const int32_t* names,
                    double* state, const double* kappa, double t0, double dt, int nsteps,
                    int negatives, double invalid_fill_value, int nthreads,
                    const obgc_gas_exchange* gas /* CO2 on DIC, or NULL */);

/* ---- negative tracers (src/Utils/negative_tracers.jl) ---- */
#define OR_MAX_GROUPS 5
#define OR_MAX_GROUP 10
/* conserved_tracers(bgc) (NutrientsPlanktonDetritus/coupling_utils.jl:1-52) as slots of `names`
 * and scale factors; returns the number of groups (nitrogen, then carbon with the carbonate
 * system).  gn[g] members, gslot/gfac [OR_MAX_GROUPS][OR_MAX_GROUP]. */
int or_conserved_groups(const obgc_npd_params* p, int n_tracers, const int32_t* names, int32_t* gn,
                        int32_t* gslot, double* gfac);
/* ScaleNegativeTracers on one cell whose tracer q is at v[q * stride] (negative_tracers.jl:250-276). */
void or_scale_cell(double* v, long stride, int ng, const int32_t* gn, const int32_t* gslot,
                   const double* gfac, double invalid_fill_value);

/* ---- ScaleNegativeTracers (src/Utils/negative_tracers.jl:250-276) ---- */
void or_scale_negatives(int64_t n, int ntr, double* const* fields, const double* scalefactors,
                        double invalid_fill_value);

/* ---- PISCES (src/Models/AdvectedPopulations/PISCES) ---- */
void or_pisces_defaults(obgc_pisces_params* p);
/* ---- air-sea gas exchange (src/Models/GasExchange) ---- */
int or_gas_exchange_defaults(int gas, obgc_gas_exchange* g);
double or_schmidt_number(const double* c, double T);
double or_transfer_velocity_660(const double* c, double u);
double or_o2_solubility(const double* A, double T, double S);
/* flux k (C_water - C_air), positive out of the ocean; u10 and air given per column */
double or_gas_exchange_flux(const obgc_gas_exchange* g, double T, double S, double DIC, double Alk, double O2,
                            double u10, double air);

double or_cbm_day_length(double coefficient, double t, double phi);
/* values [OBGC_PIS_NUM] in the PISCES tracer order, aux [OBGC_PAUX_NUM]; z the cell centre (m),
 * t the model time (s). */
double or_pisces_tendency(const obgc_pisces_params* p, int n, const double* values, const double* aux, double z, double t);
void or_pisces_tendencies(const obgc_pisces_params* p, const double* values, const double* aux, double z, double t, double* G);
void or_pisces_goc_speed(const obgc_pisces_params* p, int Nz, const double* zc, double zmxl, double zeu, double* w_faces);
double or_mixed_layer_mean(int Nz, const double* zf, const double* C, double zmxl);
int or_pisces_conserved_groups(const obgc_pisces_params* p, int32_t* gn, int32_t* gslot, double* gfac);

/* 3-D PISCES with MultiBand light, WENO5 advection of all 26 tracers, the six sinking tracers and
 * RK3; update_biogeochemical_state! before every stage (PISCES/update_state.jl:1-17: MultiBand PAR
 * from PChl + DChl, euphotic depth, mixed-layer PAR, calcite saturation). */
typedef struct or_pisces3d {
    obgc_pisces_params p;
    obgc_grid grid;              /* strides ignored: arrays are dense [Nz][Ny][Nx] */
    int32_t nbands, surface_kind;   /* surface: OBGC_SURFACE_PAR_DEFAULT or _CONSTANT */
    double kw[4], e[4], chi[4], division[4];
    double surface_value;
    double mixed_layer_depth;    /* constant zmxl (m, negative)                       */
    double mean_kappa;           /* mean mixed-layer vertical diffusivity               */
    int32_t advection, negatives;
    double invalid_fill_value;
    obgc_carbon_options carbon;
} or_pisces3d;
/* state [26][N]; u, v [N] or NULL. */
void or_pisces_step3d(const or_pisces3d* m, double* state, const double* u, const double* v, double t, double dt,
                      int nsteps, int nthreads);
/* One RK3 stage of the step that starts at t (G receives the stage's tendency, Gm holds the previous
 * stage's; start: the negative-tracer modifier first, as or_pisces_step3d applies it on entry). */
void or_pisces_stage3d(const or_pisces3d* m, double* state, const double* u, const double* v, double t, double dt,
                       int stage, double* G, const double* Gm, int start, int nthreads);
/* The auxiliary fields of the last update (for tests): PAR bands and total [4][N], zeu and mixed-layer
 * PAR [2][Nx*Ny], Omega [N]. */
void or_pisces_update_state3d(const or_pisces3d* m, const double* state, double t, double* par4, double* xy2,
                              double* omega, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
