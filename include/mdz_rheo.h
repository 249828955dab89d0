/*
 * mdz_rheo.h -- C ABI of the GB300 local-rheology library (libmdz_rheo_gb300.so).
 *
 * The library evaluates MDOODZ7.0's per-node local rheology update on one
 * GPU (sm_103a).  Every entry point takes plain pointers and sizes; no
 * MDOODZ struct crosses this boundary, so the header is usable from C, C++,
 * Python (ctypes) or any FFI.  The MDOODZ-side drop-in (the functions with the
 * reference's own signatures, which unpack `grid`/`mat_prop`/`params`/`scale`
 * into the structs below) lives in mdoodz7.0_gb300/host/mdz_rheo_mdoodz.c.
 *
 * Reference interfaces replaced (paths inside the MDOODZ7.0 tree):
 *   mdz_rheo_sweep          <- NonNewtonianViscosityGrid
 *                              MDLIB/mdoodz-private.h:423, def MDLIB/RheologyDensity.c:1131
 *   mdz_rheo_sweep_aniso    <- NonNewtonianViscosityGridAniso
 *                              MDLIB/mdoodz-private.h:437, def MDLIB/AnisotropyRoutines.c:885
 *   mdz_rheo_points         <- ViscosityConcise / ViscosityConciseAniso called per point
 *                              MDLIB/mdoodz-private.h:634-635 (callers: FD_Jacobian.c:66-67,
 *                              RheologyDensity.c:2194 GenerateDeformationMaps)
 *   (vertex fields T_s,P_s,d0_s,phi0_s)  <- InterpCentroidsToVerticesDouble
 *                              MDLIB/GridRoutines.c:108, fused into the sweep
 *   mdz_rheo_operators      <- RheologicalOperators (with FD_Jacobian.c's derivatives)
 *                              MDLIB/mdoodz-private.h:607, def MDLIB/StokesRoutines.c:75
 *   mdz_rheo_strain_rates   <- StrainRateComponents
 *                              MDLIB/mdoodz-private.h:426, def MDLIB/RheologyDensity.c:2001
 *   mdz_rheo_softening      <- CohesionFrictionDilationGrid after its P2Mastah step
 *                              def MDLIB/RheologyDensity.c:1539 (Softening :1432)
 *   mdz_rheo_shear_modulus  <- ShearModCompExpGrid, def MDLIB/RheologyDensity.c:1634
 *   mdz_rheo_marker_stress  <- UpdateParticleStress
 *                              MDLIB/mdoodz-private.h:415, def MDLIB/RheologyParticles.c:1725
 *   mdz_rheo_p2mastah       <- P2Mastah for marker arrays onto centroids or vertices
 *                              MDLIB/mdoodz-private.h:350, def MDLIB/ParticleRoutines.c:2170
 *
 * All arithmetic is IEEE binary64.  Unless a call says otherwise it is
 * synchronous (returns after the results are in the caller's buffers), like
 * the reference.
 */
#ifndef MDZ_RHEO_H
#define MDZ_RHEO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDZ_RHEO_ABI_VERSION 1
#define MDZ_MAX_PHASES 20 /* mat_prop arrays are sized [20] (MDLIB/include/mdoodz.h:152-240) */

/* ---- status codes ------------------------------------------------------
 * The reference prints a message and calls exit(); the library returns one of
 * these instead.  The drop-in maps them back to the reference's exit codes. */
#define MDZ_OK                0
#define MDZ_EINVAL           -1  /* bad argument / size */
#define MDZ_ECUDA            -2  /* CUDA runtime error */
#define MDZ_EUNSUPPORTED     -3  /* flag combination outside the implemented path */
#define MDZ_ENOMEM           -4
#define MDZ_ENOTREADY        -5  /* e.g. warm start requested without weights */
#define MDZ_EVE_ITER        -10  /* VE local iterations failed  (RheologyDensity.c:175-177, exit 0) */
#define MDZ_EGSE_ITER       -11  /* GSE local iteration failed / non-finite (:312-315, :366-368, exit 346) */
#define MDZ_ESINGULAR       -12  /* singular 3x3 plastic Jacobian (:839-841, exit 1) */
#define MDZ_EEMPTY_CELL     -13  /* cell went empty (:1274-1277, exit 345) */
#define MDZ_ENONFINITE      -14  /* Inf/NaN harmonic viscosity (:1280-1301, exit 1) */
#define MDZ_EWDISS          -15  /* negative dissipation (:1045-1050, exit 1) */
#define MDZ_EGRAIN_ZERO     -16  /* grain-size dependent creep with d=0 (:507-510, exit 1) */
#define MDZ_ELINESEARCH     -17  /* tensile line search alpha<0.01 (:868-872, exit 0) */
#define MDZ_EANISO_NAN      -18  /* aniso VE residual NaN (AnisotropyRoutines.c:543, exit 1) */
#define MDZ_EANISO_ITER     -19  /* aniso VE iterations failed (AnisotropyRoutines.c:580-583, exit 0) */
#define MDZ_ESCRATCH        -20  /* request larger than the static scratch of mdz_rheo_points_static */
#define MDZ_ESHEAR_INF      -21  /* infinite centroid shear modulus (RheologyDensity.c:1688-1690, exit 32) */
#define MDZ_EMARKER_OUT     -22  /* marker beyond the vertex grid in x (ParticleRoutines.c:1258-1266, exit 89) */

/* memory space of the field pointers handed to a sweep */
#define MDZ_MEM_HOST   0  /* host memory (drop-in mode): the library copies in and out, except
                             that arrays the device can address -- page-locked arrays mapped at
                             the same pointer, and any pageable array where the GPU reads
                             pageable memory through the host page tables (Grace-Blackwell;
                             mdz_rheo_host_access) -- are read and written in place over the
                             host link by every call but mdz_rheo_points_static, which stages
                             through its static array; MDZ_SWEEP_STAGED forces the copies where
                             a call takes flags */
#define MDZ_MEM_DEVICE 1  /* device memory of the context's GPU: no copies */

/* sweep flags */
#define MDZ_SWEEP_ASYNC      0x1  /* MDZ_MEM_DEVICE only: return after enqueue; call mdz_rheo_sync */
#define MDZ_SWEEP_WARMSTART  0x2  /* start each local Newton from the learned guess (needs weights) */
#define MDZ_SWEEP_ITERS      0x4  /* record a word per (node, phase): iterations and mechanisms (mdz_rheo_get_iterations) */
#define MDZ_SWEEP_REF_START  0x8  /* start each local Newton where the reference does (see below) */
#define MDZ_SWEEP_WARM_TILES 0x10 /* with MDZ_SWEEP_WARMSTART: evaluate the network CTA-wide on tcgen05
                                     (128-node tiles, CTA barriers per phase) instead of per warp */
#define MDZ_SWEEP_STAGED     0x20 /* MDZ_MEM_HOST: stage every array through device copies in row
                                     bands even where the GPU can address the host arrays directly */
#define MDZ_OPS_PER_NODE     0x40 /* mdz_rheo_operators: run the isotropic Newton operator one thread
                                     per node instead of compacting its plastic returns per CTA
                                     (the same bits; for comparison) */
#define MDZ_DEFAULT_POLISH   4    /* FP32 Newton steps before each FP64 local solve, by default */
/* Start descriptor of the local solves (mdz_rheo_set_warmstart): FP32 Newton steps in the
 * low byte, plus MDZ_START_DD for one Halley step evaluated in double-float (FP32 pairs)
 * after them.  The default takes both, which puts the FP64 Newton's start within its
 * stopping tolerance, so it stops at its first evaluation. */
#define MDZ_START_DD         0x100
#define MDZ_DEFAULT_START    (MDZ_DEFAULT_POLISH | MDZ_START_DD)

/* Per-(node, phase) item word recorded by MDZ_SWEEP_ITERS (mdz_rheo_get_iterations): the
 * local visco-elastic Newton's evaluations in bits 0-7 (at most 255), then the
 * mechanism switches of that local solve (RheologyDensity.c:471-483,
 * AnisotropyRoutines.c:322-326; the Peierls switch includes its temperature gate) and
 * whether it yielded (is_pl, RheologyDensity.c:663, AnisotropyRoutines.c:627); 0 for an
 * inactive phase. */
#define MDZ_MECH_CONSTANT    (1 << 8)
#define MDZ_MECH_DISLOCATION (1 << 9)
#define MDZ_MECH_PEIERLS     (1 << 10)
#define MDZ_MECH_DIFFUSION   (1 << 11)
#define MDZ_MECH_GBS         (1 << 12)
#define MDZ_MECH_GRAIN_SIZE  (1 << 13)
#define MDZ_MECH_PLASTIC     (1 << 14)  /* a plastic return is on (plast != 0 and, isotropic, step != 0) */
#define MDZ_MECH_ELASTIC     (1 << 15)
#define MDZ_MECH_YIELD       (1 << 16)  /* the point yielded: is_pl */
#define MDZ_ITEM_ITERS(w)    ((w) & 0xff)
#define MDZ_ITEM_WORD(iters, mech) ((int32_t)(((iters) > 255 ? 255 : (iters)) | (mech)))

/* ---- per-phase material table -----------------------------------------
 * The subset of `mat_prop` (MDLIB/include/mdoodz.h:152-240) that the local
 * update reads, with the same names and units (already scaled).            */
typedef struct mdz_materials {
  int    Nb_phases;
  double R;                              /* gas constant, scaled */
  /* mechanism switches */
  int    cstv[MDZ_MAX_PHASES], pwlv[MDZ_MAX_PHASES], linv[MDZ_MAX_PHASES], gbsv[MDZ_MAX_PHASES],
         expv[MDZ_MAX_PHASES], gs[MDZ_MAX_PHASES], kin[MDZ_MAX_PHASES], plast[MDZ_MAX_PHASES],
         density_model[MDZ_MAX_PHASES], phase_mix[MDZ_MAX_PHASES], phase_two[MDZ_MAX_PHASES],
         reac_soft[MDZ_MAX_PHASES], reac_phase[MDZ_MAX_PHASES], melt[MDZ_MAX_PHASES];
  /* general */
  double eta0[MDZ_MAX_PHASES], rho[MDZ_MAX_PHASES], drho[MDZ_MAX_PHASES], alp[MDZ_MAX_PHASES],
         bet[MDZ_MAX_PHASES], T0[MDZ_MAX_PHASES], P0[MDZ_MAX_PHASES], Slim[MDZ_MAX_PHASES],
         eta_vp[MDZ_MAX_PHASES], n_vp[MDZ_MAX_PHASES], T_st[MDZ_MAX_PHASES], gs_ref[MDZ_MAX_PHASES];
  /* dislocation (power law) */
  double Qpwl[MDZ_MAX_PHASES], Vpwl[MDZ_MAX_PHASES], npwl[MDZ_MAX_PHASES], mpwl[MDZ_MAX_PHASES],
         rpwl[MDZ_MAX_PHASES], Apwl[MDZ_MAX_PHASES], fpwl[MDZ_MAX_PHASES], apwl[MDZ_MAX_PHASES],
         Fpwl[MDZ_MAX_PHASES], pref_pwl[MDZ_MAX_PHASES];
  /* diffusion (linear) */
  double Qlin[MDZ_MAX_PHASES], Vlin[MDZ_MAX_PHASES], nlin[MDZ_MAX_PHASES], mlin[MDZ_MAX_PHASES],
         rlin[MDZ_MAX_PHASES], Alin[MDZ_MAX_PHASES], flin[MDZ_MAX_PHASES], alin[MDZ_MAX_PHASES],
         Flin[MDZ_MAX_PHASES];
  /* grain-boundary sliding */
  double Qgbs[MDZ_MAX_PHASES], Vgbs[MDZ_MAX_PHASES], ngbs[MDZ_MAX_PHASES], mgbs[MDZ_MAX_PHASES],
         rgbs[MDZ_MAX_PHASES], Agbs[MDZ_MAX_PHASES], fgbs[MDZ_MAX_PHASES], agbs[MDZ_MAX_PHASES],
         Fgbs[MDZ_MAX_PHASES];
  /* Peierls (exponential) */
  double Qexp[MDZ_MAX_PHASES], Sexp[MDZ_MAX_PHASES], Eexp[MDZ_MAX_PHASES], Gexp[MDZ_MAX_PHASES],
         nexp[MDZ_MAX_PHASES];
  /* paleowattmeter grain-size evolution */
  double Kpzm[MDZ_MAX_PHASES], Qpzm[MDZ_MAX_PHASES], Gpzm[MDZ_MAX_PHASES], Lpzm[MDZ_MAX_PHASES],
         cpzm[MDZ_MAX_PHASES], ppzm[MDZ_MAX_PHASES];
} mdz_materials;

/* ---- model switches and scaling ---------------------------------------
 * The `params` (MDLIB/include/mdoodz.h:49-139) and `scale` (:142-144)
 * fields the local update reads.                                           */
typedef struct mdz_model {
  int    Nx, Nz;              /* vertices; centroids are (Nx-1) x (Nz-1) */
  int    Nb_phases;
  int    step, elastic, eta_average, periodic_x, density_variations, tensile_line_search;
  int    melting, chemical_production, diffuse_X, diffuse_avg;
  double dt, min_eta, max_eta, eta_tol;
  double scale_eta, scale_L, scale_T, scale_S, scale_E;
} mdz_model;

/* ---- grid fields -------------------------------------------------------
 * Row-major flat arrays exactly as in `grid` (MDLIB/mdoodz-private.h:75-147):
 * centroid c0 = k + l*Ncx, vertex c1 = k + l*Nx.  Phase fields are arrays of
 * Nb_phases pointers (the `double**` layout of phase_perc_n etc.).
 * Fields the chosen sweep does not use may be NULL (e.g. the anisotropy
 * inputs for mdz_rheo_sweep, rho_n when density_variations==0).            */
typedef struct mdz_grid_fields {
  /* centroid inputs, (Nx-1)*(Nz-1) each */
  const double *mu_n, *T, *p_in, *d0_n, *phi0_n, *X0_n, *exxd, *ezzd, *exz_n, *sxxd0, *szzd0,
               *sxz0_n, *strain_n, *dil_n, *fric_n, *C_n, *p0_n, *T0_n, *bet_n, *div_u;
  const double *const *phase_perc_n;
  const signed char   *BCp_type;
  /* vertex inputs, Nx*Nz each */
  const double *mu_s, *X0_s, *exxd_s, *ezzd_s, *exz, *sxxd0_s, *szzd0_s, *sxz0, *strain_s,
               *dil_s, *fric_s, *C_s, *p0_s, *bet_s, *div_u_s;
  const double *const *phase_perc_s;
  const signed char   *BCg_type;
  /* anisotropy inputs (mdz_rheo_sweep_aniso only) */
  const double *d1_n, *d2_n, *angle_n, *aniso_factor_n, *d1_s, *d2_s, *angle_s, *aniso_factor_s;
  /* vertex fields interpolated from centroids (written by the sweep) */
  double *T_s, *P_s, *d0_s, *phi0_s;
  /* centroid outputs */
  double *eta_n, *eta_phys_n, *VE_n, *sxxd, *szzd, *sxz_n, *eII_el, *eII_pl, *eII_pwl, *eII_exp,
         *eII_lin, *eII_gbs, *eII_cst, *d_n, *p_corr, *div_u_el, *div_u_pl, *div_u_r, *Wtot,
         *Wel, *Wdiss, *X_n, *OverS_n, *rho_n;
  double *const *phase_eta_n;
  /* vertex outputs */
  double *sxxd_s, *szzd_s, *sxz, *eta_phys_s, *eta_s, *X_s, *VE_s;
  double *const *phase_eta_s;
} mdz_grid_fields;

/* ---- viscosity tensors of the momentum equations -----------------------
 * The coefficient fields RheologicalOperators writes (MDLIB/mdoodz-private.h:124-131). */
typedef struct mdz_operator_fields {
  /* centroids, (Nx-1)*(Nz-1) each */
  double *D11_n, *D12_n, *D13_n, *D14_n, *D21_n, *D22_n, *D23_n, *D24_n;
  double *drhodp_n; /* written by the Newton (jacobian = 1) operator only */
  /* vertices, Nx*Nz each */
  double *D31_s, *D32_s, *D33_s, *D34_s;
} mdz_operator_fields;

/* ---- sweep statistics ----------------------------------------------- */
typedef struct mdz_sweep_stats {
  uint64_t phase_calls;      /* (node, active phase) local solves */
  uint64_t newton_iters;     /* sum of VE local iterations over all phase calls */
  uint32_t max_newton_iters; /* max VE local iterations of one phase call */
  uint64_t plastic_calls;    /* phase calls that yielded (is_pl) */
  int32_t  status;           /* MDZ_OK or the first error code met */
  int64_t  error_node;       /* node of that error: centroid c0, or Nc + c1 for a vertex; -1 if none */
  double   elapsed_ms;       /* device time of the sweep kernels (CUDA events) */
  uint64_t h2d_bytes;        /* bytes moved host->device by this call (MDZ_MEM_HOST): copied, or
                                read in place from page-locked arrays */
  uint64_t d2h_bytes;        /* bytes moved device->host by this call (MDZ_MEM_HOST) */
  uint32_t kernel_launches;  /* kernels this call launched */
  uint32_t mma_fault;        /* warm start: a tensor-core wait gave up; those items used the plain start */
  uint64_t fp32_steps;       /* FP32 Newton steps taken by the starts of the local solves */
} mdz_sweep_stats;

/* ---- learned warm start ----------------------------------------------
 * A 10 (anisotropic: 12) -> 64 -> 64 -> 2 perceptron predicting, per (node, phase),
 * z = ln(eta_up / eta_ve) (eta_up: the reference's start point, the smallest isolated
 * viscosity; eta_ve: the converged visco-elastic viscosity) and a plastic indicator.
 * No reference counterpart: the reference always starts from eta_up. */
#define MDZ_MLP_IN  16  /* padded feature width */
#define MDZ_MLP_HID 64
typedef struct mdz_mlp_weights {
  int32_t n_feat;                                  /* features used: 10 or 12 */
  float   W1[MDZ_MLP_HID * MDZ_MLP_IN], b1[MDZ_MLP_HID];   /* row-major [out][in] */
  float   W2[MDZ_MLP_HID * MDZ_MLP_HID], b2[MDZ_MLP_HID];
  float   W3[2 * MDZ_MLP_HID], b3[2];
  float   x_shift[MDZ_MLP_IN], x_scale[MDZ_MLP_IN];     /* x' = (x - shift) * scale */
  float   z_shift, z_scale;                              /* z = out0 * scale + shift */
} mdz_mlp_weights;

typedef struct mdz_mlp_train_cfg {
  int32_t  epochs, batch;      /* batch: samples per Adam step (multiple of 128) */
  float    lr, lr_final;       /* cosine decay from lr to lr_final */
  float    beta1, beta2, eps;  /* Adam */
  float    w_pl;               /* weight of the plastic-indicator loss */
  uint64_t seed;               /* initialisation and sample order */
} mdz_mlp_train_cfg;

/* ---- point batches (ViscosityConcise / ViscosityConciseAniso per point) -- */
typedef struct mdz_point_inputs {
  const int32_t *phase;
  const double  *G, *T, *P, *d, *phi, *X0, *Exx, *Ezz, *Exz, *Txx0, *Tzz0, *Txz0, *strain_acc,
                *dil, *fric, *C, *P0, *T0, *beta, *div;
  const double  *lxlz, *lx2, *angle, *ani_fac; /* anisotropic points only */
  int post_process, centroid, final_update;
} mdz_point_inputs;

typedef struct mdz_point_outputs {
  double *eta;  /* return value of ViscosityConcise (eta_phys) */
  double *Txx, *Tzz, *Txz, *etaVE, *VEcoeff, *Eii_el, *Eii_pl, *Eii_pwl, *Eii_exp, *Eii_lin,
         *Eii_gbs, *Eii_cst, *d1, *X1, *OverS, *Pcorr, *rho, *div_el, *div_pl, *div_r, *Wtot,
         *Wel, *Wdiss;
  int32_t *iters;   /* VE local iterations (may be NULL) */
  int32_t *status;  /* per point MDZ_OK / error code (may be NULL) */
} mdz_point_outputs;

typedef struct mdz_rheo_ctx mdz_rheo_ctx;

/* ---- context -------------------------------------------------------- */
int         mdz_rheo_version(void);
/* sizeof() of mdz_materials, mdz_model, mdz_grid_fields, mdz_sweep_stats,
 * mdz_point_inputs, mdz_point_outputs as compiled into the library (out[0..5];
 * out[6..7] are 0), so FFI bindings can check their struct layouts. */
void        mdz_rheo_abi_sizes(size_t out[8]);
const char *mdz_rheo_status_string(int status);
/* Create a context on CUDA device `device`: one stream, device mirrors for
 * host-memory sweeps (grown on demand, kept until destroy). */
int mdz_rheo_create(int device, mdz_rheo_ctx **out);
int mdz_rheo_destroy(mdz_rheo_ctx *ctx);
/* Run the context's work on an external CUDA stream (cudaStream_t passed as
 * void*); NULL restores the context's own stream. */
int mdz_rheo_set_stream(mdz_rheo_ctx *ctx, void *stream);
/* Wait for an MDZ_SWEEP_ASYNC sweep and fetch its statistics. */
int mdz_rheo_sync(mdz_rheo_ctx *ctx, mdz_sweep_stats *stats);
/* Sweeps of host arrays (MDZ_MEM_HOST) run in bands of grid rows, so that the copies of
 * one band overlap the kernels of the others (with page-locked host arrays).  bands = 0
 * picks rows / 128, at most 16; 1 to 16 fixes the count.  Results do not depend on it. */
int mdz_rheo_set_host_bands(mdz_rheo_ctx *ctx, int bands);
/* *pageable = 1 where the context's GPU reads and writes pageable host memory (malloc,
 * new, mmap) in place through the host's page tables (the attribute
 * cudaDevAttrPageableMemoryAccessUsesHostPageTables, as on Grace-Blackwell), so that
 * MDZ_MEM_HOST calls use ordinary host arrays without copies; 0 where only page-locked
 * arrays are used in place. */
int mdz_rheo_host_access(mdz_rheo_ctx *ctx, int *pageable);

/* ---- the hot path --------------------------------------------------- */
/* NonNewtonianViscosityGrid: vertex interpolation of T, p_in, d0, phi0, then
 * every centroid and vertex: per active phase local solve, phase averaging,
 * final stress.  `mem` is MDZ_MEM_HOST or MDZ_MEM_DEVICE; `stats` may be NULL.
 * Start of the local solves: the reference starts its visco-elastic Newton at the
 * smallest isolated viscosity (RheologyDensity.c:582-592; after 10 bisection steps in
 * the anisotropic routine, AnisotropyRoutines.c:474-497).  By default the FP64 Newton
 * here starts after MDZ_DEFAULT_POLISH FP32 Newton steps from that point and one
 * double-float Halley step (MDZ_DEFAULT_START); it still iterates to the reference's
 * residual tolerance (|r| < 1e-13 Eii), so results agree with the reference to that
 * tolerance.  MDZ_SWEEP_REF_START starts exactly where the reference does (same
 * iteration counts). */
int mdz_rheo_sweep(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat,
                   const mdz_grid_fields *f, int final_update, int mem, int flags,
                   mdz_sweep_stats *stats);
/* NonNewtonianViscosityGridAniso, same conventions. */
int mdz_rheo_sweep_aniso(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat,
                         const mdz_grid_fields *f, int final_update, int mem, int flags,
                         mdz_sweep_stats *stats);
/* ViscosityConcise (aniso=0) or ViscosityConciseAniso (aniso=1) on n points (start of
 * the local solves as in mdz_rheo_sweep without flags). */
int mdz_rheo_points(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat,
                    const mdz_point_inputs *in, mdz_point_outputs *out, int64_t n, int aniso,
                    int mem);
/* RheologicalOperators (MDLIB/StokesRoutines.c:75-410): the viscosity tensors D of the
 * momentum equations from a grid that a sweep has just updated.  It reads the sweep's
 * inputs and its outputs eta_n, eta_s, phase_eta_n/_s, T_s and P_s.
 *   jacobian = 0: the Picard operator (from eta and the anisotropy fields only);
 *   jacobian = 1: the Newton operator.  Its derivatives d(eta)/dE, d(eta)/dP,
 *     d(div_pl)/dE and d(rho)/dP are central differences over 8 perturbed local solves
 *     per node and active phase (DerivativesOnTheFly_n / _s and PhaseRheologyLoop_v1,
 *     MDLIB/FD_Jacobian.c:48-323), all solved on the GPU in one launch.
 * `compressible` is params.compressible; `flags` may hold MDZ_SWEEP_REF_START, which
 * starts the perturbed solves where the reference does, and MDZ_OPS_PER_NODE.  The
 * isotropic Newton operator walks the 8 perturbations and the phases of a CTA's 128 nodes
 * in step and runs the Drucker-Prager returns of each phase's yielding items packed into
 * the CTA's first warps; MDZ_OPS_PER_NODE runs one thread per node instead, with the same
 * bits.  `mem` and `stats` as for the sweep (stats count the perturbed local solves). */
int mdz_rheo_operators(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat,
                       const mdz_grid_fields *f, mdz_operator_fields *ops, int jacobian, int compressible,
                       int aniso, int mem, int flags, mdz_sweep_stats *stats);

/* ---- strain rates from the velocity field -------------------------------
 * The arrays StrainRateComponents (MDLIB/RheologyDensity.c:2001-2097) reads and
 * writes, in the staggered layout of `grid`: u_in holds Nx*(Nz+1) x-velocity nodes
 * (u node k + l*Nx), v_in holds (Nx+1)*Nz z-velocity nodes (v node k + l*(Nx+1)).
 * wxz is written at vertices with BCg_type != 30 only; elsewhere it keeps its value. */
typedef struct mdz_strain_rate_fields {
  const double *u_in, *v_in;
  const signed char *BCp_type, *BCg_type;
  double *div_u, *exxd, *ezzd, *exz_n, *wxz_n;   /* centroids, (Nx-1)*(Nz-1) each */
  double *exz, *wxz, *exxd_s, *ezzd_s, *div_u_s; /* vertices, Nx*Nz each */
} mdz_strain_rate_fields;

/* StrainRateComponents (MDLIB/RheologyDensity.c:2001-2097, the first step of
 * UpdateNonLinearity, MDLIB/StokesRoutines.c:55-58): velocity gradients, divergence
 * and deviatoric normal strain rates at centroids, shear strain rate and spin at
 * vertices, their 4-point centroid averages, and the vertex interpolation of exxd,
 * ezzd, div_u (InterpCentroidsToVerticesDouble, MDLIB/GridRoutines.c:108-210), in one
 * launch.  dx, dz are mesh->dx, mesh->dz; out_of_plane and compressible are
 * params.out_of_plane and params.compressible; model supplies Nx, Nz and periodic_x.
 * Results are those of the reference to the last bit.  `mem` as for the sweep;
 * `flags` may hold MDZ_SWEEP_ASYNC (device memory only); `stats` may be NULL. */
int mdz_rheo_strain_rates(mdz_rheo_ctx *ctx, const mdz_model *model, double dx, double dz, int out_of_plane,
                          double compressible, mdz_strain_rate_fields *sr, int mem, int flags,
                          mdz_sweep_stats *stats);

/* ---- per-node input preparation of the sweep ---------------------------
 * The `mat_prop` fields (MDLIB/include/mdoodz.h:152-240) that Softening,
 * CohesionFrictionDilationGrid and ShearModCompExpGrid read, same names and units. */
typedef struct mdz_prep_materials {
  int    Nb_phases;
  double G[MDZ_MAX_PHASES], bet[MDZ_MAX_PHASES], alp[MDZ_MAX_PHASES];
  double C[MDZ_MAX_PHASES], phi[MDZ_MAX_PHASES], psi[MDZ_MAX_PHASES], H_c[MDZ_MAX_PHASES];
  double C_end[MDZ_MAX_PHASES], phi_end[MDZ_MAX_PHASES], psi_end[MDZ_MAX_PHASES];
  double pls_start[MDZ_MAX_PHASES], pls_end[MDZ_MAX_PHASES];
  int    phi_soft[MDZ_MAX_PHASES], psi_soft[MDZ_MAX_PHASES], coh_soft[MDZ_MAX_PHASES];
} mdz_prep_materials;

/* Grid arrays of the preparation steps (layout of mdz_grid_fields). */
typedef struct mdz_prep_fields {
  const double *const *phase_perc_n, *const *phase_perc_s;
  const signed char *BCp_type, *BCg_type;
  /* accumulated plastic strain on the grid: what P2Mastah interpolates from the markers
   * in CohesionFrictionDilationGrid (RheologyDensity.c:1558, :1595) */
  const double *strain_pl_n, *strain_pl_s;
  const double *noise_n, *noise_s;               /* read when marker_noise == 1 */
  double *fric_n, *dil_n, *C_n, *fric_s, *dil_s, *C_s;  /* softening outputs */
  double *mu_n, *bet_n, *alp, *mu_s, *bet_s;             /* shear modulus outputs */
} mdz_prep_fields;

/* CohesionFrictionDilationGrid (MDLIB/RheologyDensity.c:1539-1628) after its particle
 * interpolation: Softening (:1432-1532) of friction, dilation and cohesion against the
 * plastic strain at every centroid and vertex, arithmetic phase average, marker noise
 * on the cohesion.  The style follows params: 1 when smooth_softening == 1 (erfc form),
 * 2 when hardening_modulus == 1 (linear hardening of C), else 0 (piecewise linear).
 * Styles 0 and 2 are the reference's results to the last bit; style 1 agrees to the
 * accuracy of erfc (CUDA's on the device, the C library's in the reference).
 * Reads phase_perc_n/_s, BC flags, strain_pl_n/_s (and noise_n/_s); writes fric, dil,
 * C at centroids and vertices.  `mem`, `flags` (MDZ_SWEEP_ASYNC) and `stats` as for
 * mdz_rheo_strain_rates. */
int mdz_rheo_softening(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_prep_materials *mat,
                       mdz_prep_fields *f, int smooth_softening, int hardening_modulus, int marker_noise,
                       int mem, int flags, mdz_sweep_stats *stats);

/* ShearModCompExpGrid (MDLIB/RheologyDensity.c:1634-1755): harmonic phase averages of
 * the shear modulus G and the compressibility bet at centroids and vertices, arithmetic
 * average of the expansivity alp at centroids, and the periodic averaging of the first
 * and last vertex columns.  An infinite centroid shear modulus returns
 * MDZ_ESHEAR_INF (the reference exits with code 32).  Bit for bit the reference's.
 * Reads phase_perc_n/_s and the BC flags; writes mu_n, bet_n, alp, mu_s, bet_s. */
int mdz_rheo_shear_modulus(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_prep_materials *mat,
                           mdz_prep_fields *f, int mem, int flags, mdz_sweep_stats *stats);

/* ---- marker feedback of the sweep: UpdateParticleStress -----------------
 * The markers (`markers`, MDLIB/mdoodz-private.h:30-49) the stress update reads and
 * writes.  Inactive markers have phase -1. */
typedef struct mdz_markers {
  int64_t        n;                  /* Nb_part */
  const double  *x, *z;
  const int32_t *phase;
  double        *sxxd, *szzd, *sxz;  /* marker stresses, updated in place */
  double        *nx, *nz;            /* director, updated when anisotropy and advection are on */
} mdz_markers;

/* The grid side of UpdateParticleStress: spacing, node coordinates as the reference
 * builds them (GridRoutines.c:270-315: xg/zg vertex coordinates, Nx and Nz of them;
 * xvz/zvx the centroid coordinates with one ghost at each end, Nx+1 and Nz+1 of them;
 * xc/zc the centroid coordinates, Nx-1 and Nz-1 of them), the sweep's new and old
 * stresses, the velocities (director rotation only) and the vertex viscosity (subgrid
 * stress diffusion only). */
typedef struct mdz_marker_grid {
  double dx, dz;
  const double *xg_coord, *zg_coord, *xvz_coord, *zvx_coord;
  const signed char *BCp_type, *BCg_type;
  const double *sxxd, *szzd, *sxxd0, *szzd0;  /* centroids */
  const double *sxz, *sxz0;                   /* vertices */
  const double *u_in, *v_in;                  /* staggered velocities (layout of mdz_strain_rate_fields) */
  double *wxz;                                /* vertices; rewritten as the reference rewrites it (below) */
  const double *xc_coord, *zc_coord;          /* subgrid_diffusion 2 */
  const double *eta_phys_s;                   /* vertices; subgrid_diffusion 2 */
} mdz_marker_grid;

/* The params switches of UpdateParticleStress (MDLIB/include/mdoodz.h:49-139), and for
 * subgrid_diffusion 2 the shear modulus of every phase (mat_prop G, host memory,
 * model->Nb_phases entries). */
typedef struct mdz_marker_opts {
  int elastic, subgrid_diffusion, stress_rotation, anisotropy, advection, interp_stencil;
  const double *G;
} mdz_marker_opts;

/* UpdateParticleStress (MDLIB/RheologyParticles.c:1725-2004):
 *   - with anisotropy and advection on, the director of every active marker turns with
 *     the velocity gradients interpolated from the grid (:1784-1802);
 *   - with elastic on and subgrid_diffusion 0 or 1, every marker takes the grid's stress
 *     increments sxxd - sxxd0, szzd - szzd0 (centroids, Interp_Grid2P_centroids2) and
 *     sxz - sxz0 (vertices, Interp_Grid2P) (:1919-1966);
 *   - with elastic on and subgrid_diffusion 2 (:1811-1903), every active marker relaxes
 *     towards the old grid stress interpolated to it over its Maxwell time eta_phys_s/G
 *     (the subgrid increment), the subgrid increments go to the grid by P2Mastah, and
 *     the rest of the grid's increment comes back to the markers;
 *   - then the stress rotation of stress_rotation 1 (Jaumann) or 2 (analytical)
 *     (:1967-1992).  The reference rotates with a marker spin that its P2Mastah call
 *     fills the other way round (markers -> grid, from a zeroed marker array), so the
 *     rotation turns by zero and wxz is overwritten with zeros wherever markers reach a
 *     vertex; both are reproduced.
 * model supplies Nx, Nz, periodic_x, dt and (subgrid_diffusion 2) Nb_phases.  Results
 * are those of the reference to the last bit, except the director, whose normalisation
 * squares by multiplication where the reference calls pow (a few ulp), and subgrid
 * diffusion 2, whose P2Mastah sums run in another order (the reference's own order
 * depends on its thread count) and whose exp is CUDA's: within 1e-12 of the stress
 * scale.  A marker outside the vertex grid in x returns MDZ_EMARKER_OUT (the reference
 * exits with code 89); a non-finite increment MDZ_ENONFINITE (exit 1); a marker phase
 * outside [0, Nb_phases) with subgrid_diffusion 2, MDZ_EINVAL.  `mem`, `flags`
 * (MDZ_SWEEP_ASYNC) and `stats` as for mdz_rheo_strain_rates. */
int mdz_rheo_marker_stress(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_marker_opts *opts,
                           mdz_marker_grid *grid, mdz_markers *markers, int mem, int flags,
                           mdz_sweep_stats *stats);

/* P2Mastah (MDLIB/ParticleRoutines.c:2170-2665) for a marker array (flag 1) onto the
 * centroids (node_n, Nx-1 by Nz-1, at xc_coord/zc_coord, skipping BCp air) and/or the
 * vertices (node_s, Nx by Nz, at xg_coord/zg_coord, skipping BCg air): every active
 * marker spreads its value with the weights (1 - |X - x|/L)(1 - |Z - z|/L') over its
 * nearest node (interp_stencil 1, L = dx/2) or the 3 x 3 nodes around it (9, L = 3dx/2);
 * a node whose weight sum WM reaches 1e-30 takes sum(w v) / WM (avg 0), the harmonic
 * mean (avg 1: values 1/v, node 1/mean) or the geometric mean (avg 2: log v, exp of the
 * mean); other nodes keep their value.  With periodic_x the two ends of each vertex row
 * take their mean.  Used by CohesionFrictionDilationGrid (RheologyDensity.c:1552-1553)
 * for the plastic strain.  The reference sums per OpenMP thread, so its last bits follow
 * its thread count; these sums run in another order: results within 1e-13 of the
 * field's scale.  model supplies Nx, Nz, Nb_phases (marker phases must be below it:
 * MDZ_EINVAL) and periodic_x; grid the spacing, coordinates and BC flags; markers x, z,
 * phase and n.  `mem`, `flags` and `stats` as for mdz_rheo_strain_rates. */
int mdz_rheo_p2mastah(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_marker_grid *grid,
                      const mdz_markers *markers, const double *values, int avg, int interp_stencil,
                      double *node_n, double *node_s, int mem, int flags, mdz_sweep_stats *stats);

/* ---- allocation-free variant (no reference counterpart) ----------------
 * mdz_rheo_points on the CURRENT device without any context and without allocating:
 * no cudaMalloc / cudaFree / cudaHostAlloc and no allocating library call.  For callers
 * that must not allocate during a time step: cudaFree synchronises the whole device
 * (stalling the caller's other streams), and a caller that sizes its device memory once
 * at start-up (a solver holding most of HBM, a fixed-budget service) cannot absorb
 * allocations made inside the call.
 * Staging and statistics live in one file-scope static __device__ array of
 * MDZ_STATIC_SCRATCH_BYTES (4 MiB, 256-byte aligned) per device:
 *   bytes needed = 256 (statistics) + for MDZ_MEM_HOST, for every non-NULL array the
 *   kernel uses (phase, the 18 inputs, lxlz/lx2/ani_fac when anisotropic, every non-NULL
 *   output), n * element size rounded up to 256; for MDZ_MEM_DEVICE only the 256.
 *   strain_acc, div and angle are not read and not staged.
 * A request above the array returns MDZ_ESCRATCH before anything is enqueued (about
 * 12,000 isotropic or 11,000 anisotropic points with every input and output present,
 * host memory).
 * Nothing in the array has to start at zero: the call itself resets the statistics
 * block (counters 0, error key all ones) on `stream` before its kernel.  Stream 0 / NULL
 * is the legacy default stream.  The call is blocking: it returns after `stream` has
 * drained, with outputs (and `stats`, may be NULL) in place, so it cannot be recorded
 * into a CUDA graph.  Two calls that overlapped
 * on one device would race on the one array; calls are therefore serialised per
 * process by a lock held until the stream has drained.
 * The first call on each device looks up the array's address with
 * cudaGetSymbolAddress (that device current); make it before any stream capture
 * starts.  The address is kept for the life of the process: after a device reset
 * (cudaDeviceReset) this entry point must not be called again.  Any failure after the
 * first enqueue also waits for `stream` before the lock is released.  Inputs, outputs
 * and return codes are those of mdz_rheo_points. */
#define MDZ_STATIC_SCRATCH_BYTES (4u << 20)
int mdz_rheo_points_static(const mdz_model *model, const mdz_materials *mat, const mdz_point_inputs *in,
                           mdz_point_outputs *out, int64_t n, int aniso, int mem, void *stream,
                           mdz_sweep_stats *stats);
/* ---- many grids in one launch (no reference counterpart) ----------------
 * A batch is n device-resident grids (MDZ_MEM_DEVICE fields), each with its own model,
 * material table and size, swept together by two kernel launches, one over every grid's
 * centroids and one over every grid's vertices: each grid's centroids (vertices) are
 * cut into tiles of 128 nodes and one CTA takes one tile.  The grids'
 * arguments are folded and uploaded once, at creation; the field arrays must stay
 * valid until the batch is destroyed.  `flags` may hold MDZ_SWEEP_REF_START or
 * MDZ_SWEEP_WARMSTART (the learned warm start in every sweep of the batch, evaluated per
 * warp on the tensor cores: the context's network and start descriptor at each sweep or
 * capture; needs mdz_rheo_set_warmstart first).
 * stats->error_node counts nodes through the batch in order (grid 0's centroids, its
 * vertices, grid 1's centroids, ...). */
typedef struct mdz_rheo_batch mdz_rheo_batch;
int mdz_rheo_batch_create(mdz_rheo_ctx *ctx, int n, const mdz_model *models, const mdz_materials *mats,
                          const mdz_grid_fields *fields, int aniso, int final_update, int flags,
                          mdz_rheo_batch **out);
int mdz_rheo_batch_destroy(mdz_rheo_batch *batch);
/* One sweep of every grid of the batch: the centroid and the vertex launch on the
 * context's stream, blocking. */
int mdz_rheo_batch_sweep(mdz_rheo_batch *batch, mdz_sweep_stats *stats);
/* Capture `nsweeps` consecutive batch sweeps as one CUDA graph (replacing any earlier
 * capture).  With amp != 0 every sweep first perturbs the strain-rate inputs IN PLACE
 * (exxd, ezzd, exz_n at centroids; exxd_s, ezzd_s, exz at vertices), fused into the
 * sweep kernels' load of them (two launches per sweep, no separate pass):
 * x <- x (1 + amp u), u uniform in [-1, 1) from SplitMix64 of
 * key = sm(sm(seed ^ sweep) ^ grid), then sm(key ^ (3 node + component)), with
 * u = (h >> 11) 2^-52 - 1 (all steps rounded, no fused multiply-add).  The statistics
 * are reset once at the start of the graph and cover all of its sweeps. */
int mdz_rheo_batch_capture(mdz_rheo_batch *batch, int nsweeps, double amp, uint64_t seed);
/* Launch the captured graph on the context's stream and wait for it. */
int mdz_rheo_batch_launch(mdz_rheo_batch *batch, mdz_sweep_stats *stats);
/* CTAs per batch launch: 0 (the default) one CTA per tile; ctas > 0 a persistent grid of
 * min(ctas, tiles) CTAs that stride over the tiles (SMs x resident CTAs per SM, e.g.
 * 3 x 152, keeps every CTA resident for the whole launch).  The results are the same bits
 * either way.  Drops a captured graph: capture again before the next launch. */
int mdz_rheo_batch_set_grid(mdz_rheo_batch *batch, int ctas);

/* ---- launch-shape autotuner (no reference counterpart) -----------------
 * Times the sweep on the caller's own device-resident grid (MDZ_MEM_DEVICE fields;
 * final_update 0) in every candidate form and keeps the fastest, for later sweeps on this
 * context of the same kind: anisotropic or not, phase count, start (MDZ_SWEEP_REF_START or
 * not) and, among tuned sizes, the nearest node count (a cache keyed by those; other
 * sweeps use the last shape tuned for their kind, aniso 0/1).  Candidates, in this order:
 *   0-4   128 threads per block, 4 CTAs per SM (128 registers): one thread per node, then a
 *         grid-stride loop over 1, 2, 4 or 8 waves of the resident CTAs;
 *   5-9   the same with 64 threads per block;
 *   10    128 threads per block, one thread per node, 2 CTAs per SM (255 registers, no
 *         spills);
 *   11    persistent: one wave of resident CTAs whose warps pull 32-node chunks from a
 *         work counter (one atomic per chunk, lanes past the end retired by a ballot);
 *   12    compacting (isotropic): the CTA's threads walk their nodes' phases in step and,
 *         after each phase's visco-elastic solve, run the Drucker-Prager returns of the
 *         yielding items packed into the first threads (gathered by ballot into shared
 *         memory); the anisotropic sweep runs this candidate as one thread per node.
 * Each candidate runs one warm-up and `reps` timed sweeps; ms_out (may be NULL) receives
 * MDZ_AUTOTUNE_CANDIDATES mean kernel times and best_out (may be NULL) the chosen index.
 * No candidate changes a result bit: every node is computed by the same code, by one
 * thread, independently of the others.  `flags` may hold MDZ_SWEEP_REF_START only.  The
 * tuned sweeps overwrite the grid's outputs with the values one sweep produces.  Banded
 * host-memory sweeps take the persistent candidate's block size as one thread per node. */
#define MDZ_AUTOTUNE_CANDIDATES 13
int mdz_rheo_autotune(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat,
                      const mdz_grid_fields *f, int aniso, int flags, int reps, double *ms_out,
                      int *best_out);
/* The kernel form of that shape: 0 one thread per node or grid-stride (128 registers),
 * 1 the 255-register form, 2 the persistent work-counter form, 3 the compacting form
 * (isotropic, block 128). */
int mdz_rheo_get_launch_form(mdz_rheo_ctx *ctx, int aniso, int *form);
/* Set the shape of sweeps of this kind by hand (block 64 or 128, grid cap as above, form
 * 0/1/2; form 2 with grid_cap 0 takes one wave of resident CTAs), dropping the tuned
 * cache.  No result bit depends on it. */
int mdz_rheo_set_launch_shape(mdz_rheo_ctx *ctx, int aniso, int block, int grid_cap, int form);
/* The launch shape sweeps of this kind use now: threads per block and the grid cap
 * (0: one thread per node). */
int mdz_rheo_get_launch_shape(mdz_rheo_ctx *ctx, int aniso, int *block, int *grid_cap);

/* Per-(phase, node) item words (MDZ_ITEM_ITERS, MDZ_MECH_*) of the last sweep run with
 * MDZ_SWEEP_ITERS: out_n[p*Nc + c0], out_s[p*Nv + c1]; 0 where the phase is
 * inactive.  Host buffers. */
int mdz_rheo_get_iterations(mdz_rheo_ctx *ctx, int32_t *out_n, int32_t *out_s);

/* ---- learned warm start (no reference counterpart) --------------------- */
/* Install the network used by MDZ_SWEEP_WARMSTART (NULL removes it) and the start
 * descriptor of every FP64 local solve: FP32 Newton steps (0..64) in the low byte,
 * optionally | MDZ_START_DD (after the network's guess with MDZ_SWEEP_WARMSTART, from the
 * reference's start point otherwise; 0 = start exactly where the reference does).  The
 * default is MDZ_DEFAULT_START. */
int mdz_rheo_set_warmstart(mdz_rheo_ctx *ctx, const mdz_mlp_weights *w, int polish_iters);
/* Test hook of the tcgen05 network form (MDZ_SWEEP_WARM_TILES): the number of polls of
 * each tensor-core completion wait before the kernel gives up, records the fault
 * (mdz_sweep_stats.mma_fault), keeps the start without the network and frees its tensor
 * memory after a bounded wait for the work in flight.  0 gives up at once; a negative
 * value restores the default (2^24). */
int mdz_rheo_set_mma_poll_limit(mdz_rheo_ctx *ctx, int32_t limit);
/* A plain sweep (iso or aniso) that also records, for every (phase p, node i) item,
 * item = p * (Nc + Nv) + i (centroids first), the MDZ_MLP_IN features X[item][.] and
 * the targets Y[item][0] = ln(eta_up / eta_ve), Y[item][1] = plastic (0/1); Y[item][0]
 * is NaN for inactive items.  X and Y live in `mem` like the fields. */
int mdz_rheo_collect(mdz_rheo_ctx *ctx, const mdz_model *model, const mdz_materials *mat,
                     const mdz_grid_fields *f, int final_update, int aniso, int mem, float *X, float *Y,
                     mdz_sweep_stats *stats);
/* Train the network on n samples (X: [n][MDZ_MLP_IN], Y: [n][2], memory space `mem`) with
 * the tcgen05 training kernels.  If w->z_scale != 0 training resumes from *w, else it
 * starts from a seeded initialisation with normalisation taken from the data.  The
 * trained weights are written back to *w; loss (may be NULL) receives the mean squared
 * error of the normalised z per epoch. */
int mdz_rheo_train_mlp(mdz_rheo_ctx *ctx, const float *X, const float *Y, int64_t n, int n_feat,
                       const mdz_mlp_train_cfg *cfg, mdz_mlp_weights *w, float *loss, int mem);
/* Gradient of the training loss (mean over the n samples of (z' - z)^2 + w_pl (pl' - pl)^2,
 * z normalised by w's z_shift/z_scale) with respect to every weight, computed by the
 * same tcgen05 kernels as training, without updating: written into the W/b fields of
 * *grad (its other fields are left alone).  loss (may be NULL) receives the two sums of
 * squared errors. */
int mdz_rheo_mlp_gradient(mdz_rheo_ctx *ctx, const mdz_mlp_weights *w, const float *X, const float *Y,
                          int64_t n, float w_pl, mdz_mlp_weights *grad, float *loss, int mem);
/* Forward pass only: Yp[s] = (z, plastic indicator) for n samples. */
int mdz_rheo_mlp_predict(mdz_rheo_ctx *ctx, const mdz_mlp_weights *w, const float *X, float *Yp, int64_t n,
                         int mem);

/* ---- measurement helper ----------------------------------------------- */
/* Measured FP64 FMA throughput of `device` in TFLOP/s (a full-occupancy DFMA
 * loop timed with CUDA events).  The roofline of this FP64-bound path is
 * reported against it.  No reference counterpart. */
int mdz_rheo_measure_fp64_peak(int device, double *tflops);
/* Self-check of the device math: for n host arguments x, the table-driven exp and log
 * used on the hot path and CUDA's own exp and log, each into its host array.  No
 * reference counterpart. */
int mdz_rheo_math_selftest(int device, const double *x, int64_t n, double *fast_exp_out,
                           double *cuda_exp_out, double *fast_log_out, double *cuda_log_out);
/* Self-check of the division by a mesh spacing used by mdz_rheo_strain_rates: a[i] / b
 * by that method and by CUDA's division, for n host numerators.  No reference
 * counterpart. */
int mdz_rheo_div_selftest(int device, const double *a, int64_t n, double b, double *fast_out,
                          double *cuda_out);
/* Self-check of the quotient the local solve uses for its outputs (1/eta, 2/Tii, the
 * node's reciprocals): out[i] = r[i] / den[i] from two Newton steps on the hardware
 * reciprocal estimate (within 2 ulp of the IEEE quotient; den outside [2^-1000, 2^1000]
 * takes the IEEE division), for n host pairs.  No reference counterpart. */
int mdz_rheo_quotient_selftest(int device, const double *r, const double *den, int64_t n, double *out);
/* Self-check of the cell-index ceil used by mdz_rheo_marker_stress: ceil(q[i]) from the
 * bits of q (saturated to +-2^30 beyond that range and for NaN) and CUDA's ceil, for n
 * host arguments.  No reference counterpart. */
int mdz_rheo_ceil_selftest(int device, const double *q, int64_t n, int32_t *fast_out, double *cuda_out);
/* Self-check of the double-float arithmetic of the local solve's start: for n host
 * arguments x, out[6 i ..] = the (hi, lo) FP32 pairs of x, of exp(x) and of log(x
 * rounded to FP32) (0 where that is not a positive normal FP32 number).  No reference
 * counterpart. */
int mdz_rheo_dd_selftest(int device, const double *x, int64_t n, float *out);

#ifdef __cplusplus
}
#endif
#endif /* MDZ_RHEO_H */
