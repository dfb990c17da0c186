/*
 * starfish_gpu.h -- C ABI of libstarfish_gpu.so, the GB300 (sm_103a) hot path of
 * Starfish's ES-PIC/DSMC time step.
 *
 * The Java host reaches these entry points through JNI (or the FFM API) from
 * GPU-backed subclasses registered under the reference's own plugin names
 * (KINETIC, POISSON, DSMC, MCC).  Each entry point below names the reference
 * method it replaces (paths relative to the Starfish project root,
 * src/starfish/...).
 *
 * Conventions
 *  - Every function returns an int status: SF_OK (0) or one of SF_ERR_*.
 *    sf_last_error(ctx) gives a one-line message for the last failure.  No
 *    function exits the process or blocks without bound.
 *  - Node arrays are j-major, u = j*ni + i (Mesh.IJtoN, core/domain/Mesh.java:893-897),
 *    the order of Vec.deflate (core/common/Vec.java:165-180).  Cell arrays are
 *    j-major over (ni-1)*(nj-1) cells.
 *  - Host pointers are caller-owned and only read/written during the call.
 *    Device state (particles, fields, solver) is owned by the context.
 *  - A context is not thread-safe; all work is issued on one CUDA stream per
 *    context and every call returns after its work is complete.
 */
#ifndef STARFISH_GPU_H
#define STARFISH_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sf_ctx sf_ctx;

/* ---- status codes ---------------------------------------------------------- */
#define SF_OK 0
#define SF_ERR_ARG 1           /* invalid argument / unsupported configuration   */
#define SF_ERR_CUDA 2          /* CUDA runtime error                              */
#define SF_ERR_NOT_CONVERGED 3 /* solver hit its iteration cap (Solver.java:384)  */
#define SF_ERR_DIVERGED 4      /* NaN/Inf residual (Solver.calculateResidue 437)  */
#define SF_ERR_TIMEOUT 5       /* a bounded device wait gave up                   */
#define SF_ERR_OOM 6           /* device allocation failed / capacity exceeded    */
#define SF_ERR_STATE 7         /* call out of order (e.g. no field set yet)       */

/* ---- enumerations, numerically equal to the reference's codes ------------------ */
/* DomainModule.DomainType */
#define SF_DOMAIN_XY 0
#define SF_DOMAIN_RZ 1
#define SF_DOMAIN_ZR 2
/* Mesh.NodeType (core/domain/Mesh.java:172-173) */
#define SF_NODE_OPEN (-1)
#define SF_NODE_DIRICHLET 0
#define SF_NODE_INSULATOR 1
#define SF_NODE_INTERNAL 2
/* Mesh.DomainBoundaryType (core/domain/Mesh.java:140-141) */
#define SF_DB_OPEN (-1)
#define SF_DB_DIRICHLET 0
#define SF_DB_NEUMANN 1
#define SF_DB_PERIODIC 2
#define SF_DB_SYMMETRY 3
#define SF_DB_MESH 4
#define SF_DB_SINK 5
#define SF_DB_CIRCUIT 6
/* Mesh.Face (core/domain/Mesh.java:107-108) */
#define SF_FACE_RIGHT 0
#define SF_FACE_TOP 1
#define SF_FACE_LEFT 2
#define SF_FACE_BOTTOM 3
/* Boundary.BoundaryType (core/boundaries/Boundary.java:124-125) */
#define SF_BT_DIRICHLET 0
#define SF_BT_OPEN 1
#define SF_BT_SINK 2
#define SF_BT_VIRTUAL 3
/* Surface impact handlers (interactions/SurfaceInteraction.java:29-36).
 * SF_SURF_PASS: the boundary has no material, the particle is not stopped
 * (KineticMaterial.java:570-571). */
#define SF_SURF_PASS (-1)
#define SF_SURF_ABSORB 0
#define SF_SURF_NONE 1
#define SF_SURF_SPECULAR 2
#define SF_SURF_DIFFUSE 3
/* field selectors for sf_get_field */
#define SF_FIELD_ND 0      /* number density of a species (Material.getDen)          */
#define SF_FIELD_U 1       /* mean velocity components (KineticMaterial U/V/W)        */
#define SF_FIELD_V 2
#define SF_FIELD_W 3
#define SF_FIELD_COUNT 4   /* raw deposited weight per node, sum of w*S (no 1/V)      */
#define SF_FIELD_NODE_VOL 5 /* node volumes in use (Mesh.node_vol)                      */
#define SF_FIELD_PHI 10    /* potential (DomainModule phi)                            */
#define SF_FIELD_RHO 11    /* charge density used by the last solve                    */
#define SF_FIELD_EFI 12    /* electric field components (DomainModule efi/efj)         */
#define SF_FIELD_EFJ 13
#define SF_FIELD_NE 14     /* Boltzmann electron density                               */
/* sampled gas properties of a species (KineticMaterial.computeFields), after
 * sf_samples_compute: nd-ave, u/v/w-ave, T, t1, t2, t3, p, mpc */
#define SF_FIELD_ND_AVE 20
#define SF_FIELD_U_AVE 21
#define SF_FIELD_V_AVE 22
#define SF_FIELD_W_AVE 23
#define SF_FIELD_T 24
#define SF_FIELD_T1 25
#define SF_FIELD_T2 26
#define SF_FIELD_T3 27
#define SF_FIELD_P 28
#define SF_FIELD_MPC 29

/* ---- mesh --------------------------------------------------------------------- */
typedef struct {
  int32_t ni, nj;            /* nodes (UniformMesh)                                  */
  double x0[2];              /* origin (UniformMesh.x0)                              */
  double dh[2];              /* spacing (UniformMesh.dh)                             */
  int32_t domain_type;       /* SF_DOMAIN_*                                          */
  const int8_t* node_type;   /* ni*nj SF_NODE_* codes (Mesh.node[i][j].type)         */
  const double* bc_value;    /* ni*nj Dirichlet values (Mesh.node[i][j].bc_value) or NULL */
  const double* node_vol;    /* ni*nj node volumes (Mesh.node_vol) or NULL = computed */
  const int8_t* face_type;   /* 4*max(ni,nj) SF_DB_* codes, rows in SF_FACE_* order;
                                RIGHT/LEFT rows indexed by j, TOP/BOTTOM rows by i   */
  int32_t n_segments;        /* linear boundary segments (LinearSegment)             */
  const double* seg_xy;      /* 4 per segment: x1, y1, x2, y2                        */
  const int32_t* seg_btype;  /* SF_BT_* of the owning boundary                       */
  const int32_t* node_seg_ptr; /* ni*nj+1 CSR of Mesh.node[i][j].segments            */
  const int32_t* node_seg_idx; /* (Mesh.setNodeControlVolumes, Mesh.java:1217-1296)  */
} sf_mesh_desc;

/* Per-step totals returned by the push, as ParticleMover accumulates them
 * (KineticMaterial.java:406-413, summed over movers at :244-256), before the
 * multiplication by the species mass. */
typedef struct {
  double n_sum;        /* sum of mpw over surviving particles                 */
  double p_sum[3];     /* sum of mpw*v                                         */
  double e_sum;        /* sum of mpw*|v| (Vec.mag3, as in the reference)        */
  double boundary_charge; /* sum of mpw*q over absorbed particles (SourceModule.boundary_charge) */
  int64_t np;          /* particles alive after the step                        */
  int64_t n_removed;   /* particles removed this step                           */
  int64_t n_slow;      /* particles that took the exact surface/exit path       */
  int64_t n_bounce_limited; /* particles that used all 10 bounces               */
} sf_push_stats;

/* Creates a context on CUDA device `device` for one uniform mesh.
 * Replaces: Mesh/UniformMesh set-up as seen by KineticMaterial and Solver
 * (UniformMesh.java:55-72, Mesh.initNodes 364-402, Solver.init 153-189). */
int sf_ctx_create(const sf_mesh_desc* mesh, int device, sf_ctx** out);
int sf_ctx_destroy(sf_ctx* ctx);
/* Seed of all random streams of the context (Starfish.random, core/common/Starfish.java:238,
 * which <starfish randomize="true"> reseeds at :647); restarts the stream counters.  The
 * default seed is fixed, so runs repeat unless a seed is set. */
int sf_ctx_set_seed(sf_ctx* ctx, uint64_t seed);
/* Last error message of a context (or of the last failed sf_ctx_create when ctx is NULL). */
const char* sf_last_error(const sf_ctx* ctx);
/* Library version string. */
const char* sf_version(void);

/* Host-side helper: per-node lists of the segments whose box test passes, as
 * Mesh.setNodeControlVolumes builds node[i][j].segments (core/domain/Mesh.java:1217-1296).
 * Call with ptr == idx == NULL to get *nnz; then ptr has ni*nj+1 and idx *nnz entries.
 * Needs no GPU.  A Java host passes its own lists instead. */
int sf_build_node_segments(int32_t ni, int32_t nj, const double* x0, const double* dh,
                           int32_t n_segments, const double* seg_xy, int32_t* ptr, int32_t* idx,
                           int64_t* nnz);

/* ---- species and particles ------------------------------------------------- */
/* Registers a kinetic species (KineticMaterial ctor; mass in kg, charge in C,
 * spwt = specific weight Material.spwt0).  capacity: maximum particles held.
 * nd_back: background density added after the scatter (Material.java:618-632). */
int sf_species_add(sf_ctx* ctx, double charge, double mass, double spwt, int64_t capacity,
                   double nd_back, int32_t* sid);
/* Automatic cell sort every `interval` pushes (default 16; 0 = only explicit sorts).
 * Sorting keeps the deposit's shared-memory tiles compact and drops removed slots. */
int sf_species_set_sort_interval(sf_ctx* ctx, int32_t sid, int32_t interval);
/* Key of the automatic sort: blocks of `cells` x `cells` cells (1, 2, 4, 8 or 16; default 8)
 * inside 16x16-cell tiles.  Coarser blocks make the sort cheaper; the push's locality is
 * that of a run of sorted particles, about the same for blocks up to 8 cells.  Explicit
 * sorts (sf_particles_sort) and the DSMC binning always sort by exact cell.  No reference
 * counterpart (the reference keeps per-cell particle lists). */
int sf_species_set_sort_block(sf_ctx* ctx, int32_t sid, int32_t cells);
/* Surface handler of the boundary owning segment `seg` for this species
 * (MaterialInteraction list, Material.performSurfaceInteraction, Material.java:279-336).
 * vth: boundary thermal speed for SF_SURF_DIFFUSE (Boundary.getVth); c_rest, c_accom:
 * MaterialInteraction coefficients.  Default for every segment: SF_SURF_ABSORB. */
int sf_species_set_surface(sf_ctx* ctx, int32_t sid, int32_t seg, int32_t model, double vth,
                           double c_rest, double c_accom);
/* Species change at a segment (SurfaceInteraction.java:128-142, 175-193, the product
 * material of MaterialInteraction): a particle of sid that hits seg with model SPECULAR or
 * DIFFUSE is removed, and (int)(spwt_sid / spwt_product + rnd) particles of product_sid
 * start from the hit point (the reference's ParticleListSource, emitted with the 1e-6 dt
 * push off and the -dt/2 rewind): specular ones with the reflected velocity, diffuse ones
 * each with its own cosine-law direction and a speed from vth_product (the product's
 * thermal speed at the wall) and the segment's c_rest, c_accom.  Products carry their
 * species' weight.  product_sid = -1 clears it.  Products past the product's capacity
 * make sf_push_deposit return SF_ERR_OOM. */
int sf_species_set_surface_product(sf_ctx* ctx, int32_t sid, int32_t seg, int32_t product_sid,
                                   double vth_product);
/* Appends particles from physical positions (KineticMaterial.addParticle, KineticMaterial.java:759-802):
 * lc = XtoL(pos), clamped to the mesh; if rewind != 0 the velocity is rewound by -dt/2
 * with the current electric field (needs sf_set_efield / a Poisson solve first).
 * pos, vel: n*3 doubles; mpw: n weights (Particle.mpw) or NULL (= spwt).  A species of
 * uniform weight takes only mpw = spwt; one switched to per-particle weights
 * (sf_species_set_weighted) takes any 0 < mpw <= spwt. */
int sf_particles_append(sf_ctx* ctx, int32_t sid, int64_t n, const double* pos, const double* vel,
                        const double* mpw, int32_t rewind, double dt);
/* Per-particle weights (Particle.mpw, KineticMaterial.java:1207-1282) for a species:
 * switched on before its first particle; the species weight spwt is then the largest
 * weight a particle may carry.  The push deposits, moments, totals and surface sums scale
 * by mpw / spwt; DSMC takes each pair's weights (Boyd's update, the collided-weight sum)
 * and MCC each particle's (S, the weight sum, the ion count; the second electron inherits
 * it); sources and surface products enter at spwt.  Batched instances take weighted
 * and uniform species side by side. */
int sf_species_set_weighted(sf_ctx* ctx, int32_t sid, int32_t on);
/* sf_particles_append_lc with per-particle weights mpw (n; a weighted species). */
int sf_particles_append_lc_w(sf_ctx* ctx, int32_t sid, int64_t n, const double* lc, const double* vel,
                             const double* mpw);
/* The weights (mpw) of the particles sf_particles_download returns, in the same order. */
int sf_particles_download_weights(sf_ctx* ctx, int32_t sid, int64_t cap, double* mpw, int64_t* n_out);
/* Appends particles given logical coordinates (Particle.lc, n*2) instead of positions;
 * no rewind.  Used to load identical state into the GPU and the reference. */
int sf_particles_append_lc(sf_ctx* ctx, int32_t sid, int64_t n, const double* lc,
                           const double* vel);
/* Number of particles currently held (alive). */
int sf_particles_count(sf_ctx* ctx, int32_t sid, int64_t* np);
/* Copies particles to the host in storage order: lc (n*2), vel (n*3); dead slots are
 * skipped.  cap = capacity of the host arrays; *n_out = particles written. */
int sf_particles_download(sf_ctx* ctx, int32_t sid, int64_t cap, double* lc, double* vel,
                          int64_t* n_out);
/* Counting sort of a species by cell; drops removed particles (the cell binning of
 * DSMC.perform(mesh), DSMC.java:194-231, done once for all users). */
int sf_particles_sort(sf_ctx* ctx, int32_t sid);
/* Removes all particles of a species. */
int sf_particles_clear(sf_ctx* ctx, int32_t sid);

/* Maxwellian boundary source on one straight segment (x1, y1, x2, y2), sampled on the
 * device: MaxwellianSource.sampleParticle (sources/MaxwellianSource.java:93-125) with the
 * particle count of Source.regenerate (core/source/Source.java:123-134), the 1e-6 dt
 * push off the surface of Source.sampleKinetic (:167-198) and the -dt/2 velocity rewind
 * of KineticMaterial.addParticle (KineticMaterial.java:776-796).  The segment normal
 * (-dy, dx)/L gives the drift direction.  den: density (m^-3), temp (K), v_drift (m/s).
 * *rem carries the fractional particle count between calls.  *n_added: particles added;
 * with n_added NULL the call returns once the draws are queued: draw k takes the k-th
 * slot behind the species' particles, and a draw landing outside the mesh leaves its slot
 * removed (counted like a push's removals, as after SF_PUSH_NOWAIT). */
int sf_source_maxwellian(sf_ctx* ctx, int32_t sid, const double* seg_xy, double den, double v_drift,
                         double temp, double dt, double* rem, int64_t* n_added);
/* UniformSource on one straight segment (sources/UniformSource.java:36-80): mass flow rate
 * mdot (kg/s) with the particle count of Source.regenerate; particles at random points of
 * the segment (area-weighted in RZ / ZR), velocity normal * v_drift with no thermal spread;
 * the push off the surface, the rewind and a null n_added as sf_source_maxwellian. */
int sf_source_uniform(sf_ctx* ctx, int32_t sid, const double* seg_xy, double mdot, double v_drift,
                      double dt, double* rem, int64_t* n_added);
/* VolumePreloadSource (sources/VolumePreloadSource.java:44-66) through VolumeSource
 * (core/source/VolumeSource.java:63-170): in every cell ceil(den cellVol / spwt) - 1
 * particles (when that number exceeds spwt) uniform in the cell, Maxwellian at
 * max(temp, 50 K) (Utils.SampleMaxw3D with its factor 1.2); points inside solid
 * boundaries (BoundaryModule.isInternal) are not added; the 1e-6 dt push off and the
 * -dt/2 rewind of addParticle.  *n_added: particles added. */
int sf_source_preload(sf_ctx* ctx, int32_t sid, double den, double temp, double dt, int64_t* n_added);

/* ---- fields ----------------------------------------------------------------- */
/* Sets the electric field used by the push (DomainModule efi/efj, FP64 host -> FP32 device). */
int sf_set_efield(sf_ctx* ctx, const double* efi, const double* efj);
/* Copies a node field to the host (FP64, ni*nj). */
int sf_get_field(sf_ctx* ctx, int32_t field, int32_t sid, double* out);

/* ---- push + scatter ---------------------------------------------------------- */
/* One time step of KineticMaterial.updateFields() for one species on one mesh:
 * ParticleMover.run (KineticMaterial.java:299-422) -- E gather, v += q/m E dt, move,
 * ProcessBoundary (:471-750) surface hits and domain exits -- followed by the node
 * scatter of updateFields(md) (:168-197) into a deterministic int64 fixed-point
 * grid and the density nd = sum(w S)/V + nd_back.
 * flags: SF_PUSH_STATS computes sf_push_stats (reads vz); SF_PUSH_MOMENTS also
 * deposits the u/v/w moments.  stats may be NULL.
 * SF_PUSH_NOWAIT: return once the push is queued on the context's stream instead of
 * waiting for it (ignored with SF_PUSH_STATS or when a surface of the species emits
 * products, which need this push's results on the host).  The removed-particle count
 * stays on the device until the next call on the species that needs it (any entry point
 * but the push itself), which waits for the stream first; stats, if given, is zeroed
 * with np, n_removed, n_slow and n_bounce_limited = -1.  Work queued after it on the
 * context's stream (sf_poisson_nl, sf_get_field, the next push) sees its results.  A
 * kernel error of a push that did not wait is reported by a later call. */
#define SF_PUSH_STATS 1
#define SF_PUSH_MOMENTS 2
#define SF_PUSH_SAMPLE 4   /* also KineticMaterial.updateSamples after the push (implies MOMENTS) */
#define SF_PUSH_NOWAIT 8
int sf_push_deposit(sf_ctx* ctx, int32_t sid, double dt, int32_t flags, sf_push_stats* stats);
/* Particle-steps pushed for the species since it was created: the sum over its
 * sf_push_deposit / sf_push_deposit_noalloc calls of the particles alive when the push
 * began (batched steps not included).  Waits for the context's stream.  No counterpart
 * in the reference (its step log prints np per step). */
int sf_species_particle_steps(sf_ctx* ctx, int32_t sid, int64_t* particle_steps);
/* Velocity sampling (KineticMaterial.updateGasProperties, KineticMaterial.java:1553-1671).
 * sf_samples_clear (clearSamples, :1509-1530) zeroes the running sums; its first call sets
 * up the species' sampling buffers (allocates).  Each sf_push_deposit with SF_PUSH_SAMPLE
 * then adds the post-push scatter of w, w v, w v^2 and the macroparticles per cell
 * (updateSamples, :1570-1595).  sf_samples_compute (computeFields, :1606-1671) derives
 * the SF_FIELD_ND_AVE..SF_FIELD_MPC fields; T_init is used where nothing was sampled
 * (Material init_vals.T).  *num_samples (may be NULL) receives the sample count. */
int sf_samples_clear(sf_ctx* ctx, int32_t sid);
int sf_samples_compute(sf_ctx* ctx, int32_t sid, double T_init, int64_t* num_samples);
/* sf_push_deposit without any device allocation; no counterpart in the reference.
 * For hosts that must not have the library call cudaMalloc while they step (their own
 * caching allocator already holds the device memory, or their device footprint is
 * fixed at start-up): the push's per-call scratch -- slow-path queue, event counters,
 * partial sums -- lives in a static __device__ array of the library instead of the
 * context's buffers.  Same arguments, results and errors as sf_push_deposit, plus:
 *  - every call waits for its work; SF_PUSH_NOWAIT is rejected with SF_ERR_ARG;
 *  - the species may hold at most 2^21 (2,097,152) particle slots (live + removed
 *    since the last sort); a larger species is rejected with SF_ERR_ARG;
 *  - the first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) and caches it for the life of the process; make that first
 *    call before any stream capture.  A device reset (cudaDeviceReset) discards the
 *    array and leaves the cached address stale, so a host that resets a device must
 *    not call this entry point again in that process;
 *  - every call, from every context on the device, shares the one array: calls whose
 *    GPU work overlaps (other threads, other contexts' streams) race on it.  Calls
 *    from one thread are safe, since each call waits for its own work to finish. */
int sf_push_deposit_noalloc(sf_ctx* ctx, int32_t sid, double dt, int32_t flags, sf_push_stats* stats);
/* Surface flux / mass deposit accumulated by the push since the last reset, per
 * segment and split over the segment ends exactly like the Field1D scatter of
 * Material.addSurfaceMomentum / addSurfaceMassDeposit (Material.java:759-796):
 * out arrays hold 2 doubles per segment (weight at the start / end node). */
int sf_get_surface_flux(sf_ctx* ctx, int32_t sid, double* flux, double* deposit);
int sf_reset_surface_flux(sf_ctx* ctx, int32_t sid);

/* ---- field solve ------------------------------------------------------------ */
/* Parameters of the nonlinear Poisson solve with Boltzmann electrons
 * (PoissonSolver, pic/PoissonSolver.java:49-107; defaults SolverModule.java:55-87). */
typedef struct {
  double n0;        /* reference electron density (m^-3), PoissonSolver.den0            */
  double kTe0;      /* electron temperature (eV), PoissonSolver.kTe0                    */
  double phi0;      /* reference potential (V), PoissonSolver.phi0                      */
  double eps;       /* permittivity, Constants.EPS0 * eps_r                             */
  double tol;       /* target FP64 residual ||R||_2 / N (LinearSolverGS metric, :111-125) */
  int32_t max_it;   /* cap on Newton / refinement iterations                            */
  int32_t cycles;   /* PCG iterations (one V-cycle each) per Newton step; <= 0: 4       */
  int32_t use_learned; /* 1: start from the learned predictor when it is trained;
                          2: the network as a coarse correction inside the PCG: the first
                          preconditioner application of the first Newton step is
                          e + V(r - J e), e the network's estimate of J^-1 r; every
                          converged solve in this mode trains it on its first residual */
  int32_t linear;   /* 1: linear Poisson (no electron term), PoissonSolver linear_mode  */
} sf_poisson_params;

typedef struct {
  int32_t newton_it;        /* outer (FP64 residual) iterations taken                  */
  int32_t vcycles;          /* inner multigrid cycles                                   */
  double residual;          /* final ||R||_2 / N (FP64)                                  */
  double residual_inf;      /* final max |R|                                             */
  double initial_residual;  /* ||R||_2 / N of the initial guess                          */
  double ms;                /* device time of the solve (CUDA events)                    */
} sf_solve_stats;

/* SolverModule.updateRho (core/solver/SolverModule.java:144-171): rho = sum over the
 * context's kinetic species of charge * nd, on the device. */
int sf_update_rho(sf_ctx* ctx);
/* Replaces the Dirichlet values (BoundaryModule.updateBoundaries -> DomainModule.updateBCvalues,
 * used for time-varying electrodes).  bc: ni*nj. */
int sf_set_bc_values(sf_ctx* ctx, const double* bc);
/* PoissonSolver.update -> solvePotentialNL -> Solver.solveNonLinearNR
 * (PoissonSolver.java:110-252, Solver.java:293-387): solves
 *   A phi = -rho/eps + (e n0/eps) exp((phi - phi0)/kTe)     (non-fixed rows)
 * to ||R||_2/N < tol in FP64: Newton on the Boltzmann term with FP64 residuals and
 * updates, each correction from FP32 geometric multigrid V-cycles.  rho: host charge
 * density (ni*nj) or NULL to use the device rho (sf_update_rho).  phi: host initial
 * guess and result, or NULL to keep the potential on the device (the previous solution
 * is then the initial guess).  Returns SF_ERR_NOT_CONVERGED / SF_ERR_DIVERGED as
 * Solver.java:384-385 and :437-439 report them.  XY, RZ and ZR meshes: on RZ/ZR, A is
 * the reference's axisymmetric FVM operator (face fluxes weighted by the face radius over
 * the node volume 2 pi r dA); the learned modes (use_learned) take XY meshes only. */
int sf_poisson_nl(sf_ctx* ctx, const sf_poisson_params* prm, const double* rho, double* phi,
                  sf_solve_stats* stats);
/* PotentialSolver.updateGradientField (pic/PotentialSolver.java:56-70): E = -grad(phi)
 * (Solver.evaluateGradient, Solver.java:789-814), kept on the device for the push and
 * optionally copied to efi/efj (ni*nj each, may be NULL). */
int sf_efield(sf_ctx* ctx, double* efi, double* efj);
/* BoltzmannElectronsMaterial.electronModelBoltzmann (BoltzmannElectronsMaterial.java:179-215):
 * n_e = max(1, n0 exp((phi - phi0)/kTe)) into ne (ni*nj, may be NULL: device only). */
int sf_boltzmann(sf_ctx* ctx, double* ne);

/* ---- learned warm start of the Poisson solve (no reference counterpart) -------- */
/* A 4-level U-Net (base_channels 16 or 32, doubling per level; BF16 weights and
 * activations, FP32 accumulation) on the mesh coarsened by `down` (1..8; (n-1)/down
 * must be a multiple of 8 and >= 16 in both directions).  From the change of rho and of
 * the Dirichlet values since the last converged solve (and the previous potential) it
 * predicts the change of phi; sf_poisson_nl with use_learned = 1 and phi = NULL starts
 * from phi_prev + prediction when that start has the lower FP64 residual, and still
 * iterates to the same tolerance.  While training is on, converged sf_poisson_nl calls
 * add Adam steps on the new pairs. */
int sf_unet_init(sf_ctx* ctx, int32_t base_channels, int32_t down, uint64_t seed);
/* Training on/off, Adam learning rate, Adam steps per training pair, and the thinning
 * of online training: one training pair every `every` converged solves. */
int sf_unet_set_training(sf_ctx* ctx, int32_t on, double lr, int32_t iters_per_sample, int32_t every);
/* Last training loss (MSE of the scaled change), pairs trained on, device ms spent
 * training, predictions used as the start of a solve and predictions rejected because
 * their FP64 residual was not below that of the previous potential (any pointer may be
 * NULL). */
int sf_unet_stats(sf_ctx* ctx, double* last_loss, int64_t* samples, double* train_ms, int64_t* used,
                  int64_t* rejected);
/* Gradient checking: runs the network on x (Hn*Wn*16 floats, NHWC, Hn = (nj-1)/down,
 * Wn = (ni-1)/down) into pred (Hn*Wn); with dpred given, back-propagates it and writes
 * the parameter gradients into grads, flattened per layer (conv weight [co][ky][kx][ci],
 * conv bias, ..., head weight, head bias; encoder convs first, then decoder, then head).
 * *nparams receives the parameter count (x may be NULL to query it only). */
int sf_unet_debug(sf_ctx* ctx, const float* x, const float* dpred, float* pred, float* grads, int64_t* nparams);
/* Reads (get) and/or replaces (set) the FP32 master parameters, same flattening. */
int sf_unet_params(sf_ctx* ctx, float* get, const float* set);
/* The network's 3x3 convolutions (forward and backward-data) run on the tcgen05 tensor
 * cores (TMA loads, accumulators in tensor memory) wherever the grid rows are 16, 32, 64
 * or a multiple of 128 nodes; on = 0 runs them all on the mma.sync kernels instead (the
 * two paths are compared in the tests).  A tensor-core pipeline that stalls gives up
 * after 2 s and the next call returns SF_ERR_TIMEOUT.  *tc_convs: convolutions run on
 * the tcgen05 path so far. */
int sf_unet_set_tensor_cores(sf_ctx* ctx, int32_t on);
int sf_unet_tensor_core_stats(sf_ctx* ctx, int64_t* tc_convs);
/* Failure-detection check of the tensor-core pipeline: runs one small convolution whose
 * copies are never issued, so that its first wait runs out (after 20 ms); the CTAs record
 * the failure, free their tensor memory and return.  Returns SF_ERR_TIMEOUT when that
 * happened (the context stays usable), SF_ERR_STATE if the timeout was not reported.
 * Needs no U-Net. */
int sf_unet_tensor_core_wait_test(sf_ctx* ctx);

/* ---- batches of independent instances (no reference counterpart) --------------- */
/* Many independent cases (contexts of different mesh sizes and particle counts, one
 * kinetic species each, XY meshes) advanced together.  One sf_batch_step does, for all
 * instances: the Maxwellian inlet sources, the push + scatter (one launch over every
 * instance's particles, the device phase replayed as one CUDA graph), then per instance
 * rho, the Poisson-Boltzmann solve and E, issued from `threads` host threads so that the
 * instances' solves overlap on the GPU.  Instances are cell-sorted every 16 steps.  The
 * first steps tune the push launch shape and the PCG iterations per Newton step per
 * mesh-size bucket (sf_batch_tuning).  The contexts stay owned by the caller and must
 * not be used by other calls while a batch step runs; between steps their usual entry
 * points work. */
typedef struct sf_batch sf_batch;
typedef struct {
  int64_t particles;         /* live particles over all instances after the step          */
  double device_phase_ms;    /* sources + push + deposit of all instances (CUDA events)    */
  double solve_ms_sum;       /* device time of the instances' Poisson solves, summed       */
  double solve_ms_max;       /* ... and the longest one                                    */
  double newton_it_mean;     /* Newton steps per solve                                     */
  int32_t newton_it_max;     /* most Newton steps of any instance in this step             */
  int32_t capacity_overflow; /* a source hit an instance's capacity (step returns SF_ERR_OOM) */
} sf_batch_stats;
int sf_batch_create(sf_ctx** ctxs, const int32_t* sids, int32_t n, int32_t threads, sf_batch** out);
int sf_batch_destroy(sf_batch* b);
const char* sf_batch_last_error(const sf_batch* b);
/* MaxwellianSource on a straight segment for instance i (as sf_source_maxwellian). */
int sf_batch_set_source(sf_batch* b, int32_t i, const double* seg, double den, double v_drift, double temp);
int sf_batch_step(sf_batch* b, double dt, const sf_poisson_params* prm, sf_batch_stats* stats);
/* Chosen push blocks per SM and exact-path blocks per SM (-1 while tuning), and PCG
 * iterations per Newton step for meshes of < 4096, < 16384 and more nodes (-1 while tuning). */
int sf_batch_tuning(const sf_batch* b, int32_t* blocks_per_sm, int32_t* slow_blocks, int32_t* cycles_by_bucket);

/* ---- collisions ------------------------------------------------------------- */
/* Cross-section models (interactions/Sigma.java:24-195, collisions/SigmaPlus.java:38-76) */
#define SF_SIGMA_CONST 0    /* sigma = c0                                         */
#define SF_SIGMA_INV 1      /* sigma = c0 / g                                     */
#define SF_SIGMA_POLY 2     /* c0 + c1 g + c2 g^2 + c3 g^4 (the reference's g *= g) */
#define SF_SIGMA_LN 3       /* sigma = (c0 + c1 ln g)^2                           */
#define SF_SIGMA_BIRD463 4  /* VHS, Bird eq. 4.63                                 */
typedef struct {
  int32_t model;      /* SF_SIGMA_*                                              */
  double c[4];        /* coefficients of CONST / INV / POLY / LN                 */
  double diam;        /* BIRD463: molecular diameter of the species (Material.diam) */
  double T_ref;       /* BIRD463: reference temperature (Material.ref_temp)       */
  double omega;       /* BIRD463: viscosity-temperature index                     */
  double vss_alpha;   /* scattering: 1 = VHS (isotropic), else VSS                */
} sf_sigma;

/* DSMC.perform for a same-species pair (collisions/DSMC.java:162-454): cell binning
 * (a counting sort of the species), then per cell the NTC selection count
 * nsel = (n1 w / Vc) n2 dt (sigma g)max / 2 + rem, random pairs accepted with
 * sigma(g) g / (sigma g)max, and the elastic VHS/VSS scattering of ModelElastic.
 * Every ordered pair of two distinct particles of a cell is an equally likely
 * candidate, as in the reference; the candidates of one parallel round share no
 * particle.  dt: frequency * dt of the reference.  sig_cr_max0: initial (sigma g)max of
 * every cell (DSMC element sig_cr_max, default 1e-16).  *n_coll: collisions performed;
 * with n_coll NULL the call returns once the collisions are queued on the context's
 * stream (the per-cell sums of sf_dsmc_get_counts hold them). */
int sf_dsmc(sf_ctx* ctx, int32_t sid, const sf_sigma* sigma, double dt, double sig_cr_max0,
            int64_t* n_coll);
/* DSMC.perform for the pair="mat1,mat2" of two kinetic species (DSMC.java:259-453):
 * both species are binned; nsel = (n1 w1 / Vc) n2 dt (sigma g)max / (Pab + (w2/w1) Pba),
 * doubled for two species, + rem, with Boyd's Pab = min(1, w2/w1), Pba = min(1, w1/w2);
 * each candidate is one uniform particle of each species; ModelElastic with the reduced
 * masses, and when the weights differ each particle's velocity changes with probability
 * w_other / w_self (Boyd 1996).  sigma1 holds the cross-section model and coefficients
 * and mat1's diameter, reference temperature, viscosity index and VSS alpha; sigma2
 * holds mat2's (its model and coefficients are not used); Bird 4.63 takes
 * d = d1 + d2 over 4 (SigmaBird463.init), the mean T_ref and omega, and vss_inv =
 * (1/alpha1 + 1/alpha2) / 2.  sid1 == sid2 is sf_dsmc (sigma2 may be NULL). */
int sf_dsmc_pair(sf_ctx* ctx, int32_t sid1, int32_t sid2, const sf_sigma* sigma1, const sf_sigma* sigma2,
                 double dt, double sig_cr_max0, int64_t* n_coll);
/* Per-cell collision sums accumulated by sf_dsmc ((ni-1)*(nj-1) each, j-major):
 * count (col-count-sum) and weight (col-real-sum, 0.5 (w1 + w2) per collision),
 * DSMC.java:241-247,344. */
int sf_dsmc_get_counts(sf_ctx* ctx, int32_t sid, double* count_sum, double* real_sum);
/* The same sums for the pair (sid1, sid2) of sf_dsmc_pair. */
int sf_dsmc_pair_get_counts(sf_ctx* ctx, int32_t sid1, int32_t sid2, double* count_sum, double* real_sum);
/* Target (background) material of MCC: mass and node fields density, mean velocity and
 * temperature (Material.getDen / getUAve.. / getT), ni*nj each; u, v, w may be NULL (0). */
int sf_mcc_set_target(sf_ctx* ctx, double mass, const double* den, const double* u, const double* v,
                      const double* w, const double* temp);
/* MCC.perform (collisions/MCC.java:167-221) for a kinetic source species against the
 * target: P = 1 - exp(-sigma(g) g dt n_t) with g from the target's mean velocity; on a
 * collision a Maxwellian target particle is drawn (Material.sampleMaxwellianVelocity)
 * and the source velocity is set by model SF_MCC_MEX (elastic, MCC.java:242-285) or
 * SF_MCC_CEX (charge exchange, :287-297). */
#define SF_MCC_MEX 0
#define SF_MCC_CEX 1
#define SF_MCC_IONIZATION 2
int sf_mcc(sf_ctx* ctx, int32_t sid, int32_t model, const sf_sigma* sigma, double dt, int64_t* n_coll);
/* MCC.perform with ModelIonization (MCC.java:304-356): electrons (species sid) against the
 * neutral target.  On a collision the electron loses ionization_energy (eV) and keeps a
 * uniform random share of the rest, with an isotropic direction; a second electron with
 * the same speed (the reference draws its speed from the first share too) is appended to
 * sid, and (int)(spwt_sid / spwt_product + rnd) ions of product_sid, Maxwellian at the
 * target temperature (100 K where it is <= 0), at the same place.  New particles get the
 * -dt/2 rewind of addParticle.  The created product weight is summed into the delta-N
 * field (sf_mcc_get_sums); the caller removes it from its target density (the
 * reference's KineticMaterial.deleteMass).  Products past a species' capacity are
 * dropped and the call returns SF_ERR_OOM.  *n_electrons / *n_ions: created. */
int sf_mcc_ionization(sf_ctx* ctx, int32_t sid, int32_t product_sid, const sf_sigma* sigma,
                      double ionization_energy, double dt, int64_t* n_coll, int64_t* n_electrons,
                      int64_t* n_ions);
/* Sums accumulated by every MCC call since the target was set or the last reset, ni*nj
 * node fields each (any pointer may be NULL): S, the target's energy term mpw (E1 - E2) /
 * (dt V) with E = 0.5 m |v| as in MCC.java:204-210, scattered like Field2D.scatter;
 * count_sum and real_sum (collisions and collided weight at node (int) lc, MCC.java:
 * 213-218); delta_n (product weight created by ionization at node (int) lc). */
int sf_mcc_get_sums(sf_ctx* ctx, double* S, double* count_sum, double* real_sum, double* delta_n,
                    int32_t reset);

/* ---- measurement ---------------------------------------------------------- */
/* The CUDA stream (cudaStream_t) all work of the context is issued on. */
int sf_ctx_get_stream(sf_ctx* ctx, void** stream);
/* Per-kernel CUDA-event timing on the context stream (off by default).  When on,
 * each hot kernel launch is bracketed by events and its device time accumulated
 * under its name ("push", "push_slow", "sort", "finalize", "poisson_residual", ...). */
int sf_timing_enable(sf_ctx* ctx, int32_t on);
int sf_timing_get(sf_ctx* ctx, const char* kernel, double* total_ms, int64_t* launches);
int sf_timing_reset(sf_ctx* ctx);
/* Number of kernels this context has launched since creation (or the last reset). */
int sf_launch_count(sf_ctx* ctx, int64_t* launches, int32_t reset);

#ifdef __cplusplus
}
#endif
#endif /* STARFISH_GPU_H */
