/*
 * horses3d_gb300 -- C ABI of the GB300 (sm_103a) compressible Navier-Stokes DGSEM
 * right-hand side and Williamson low-storage RK3 update.
 *
 * The boundary sits where HORSES3D's time integrator calls the spatial operator:
 *
 *   dg_rhs        replaces ComputeTimeDerivative
 *                 (Solver/src/NavierStokesSolver/SpatialDiscretization.f90:227-320,
 *                  interface ComputeTimeDerivative_f in
 *                  Solver/src/libs/discretization/DGSEMClass.f90:78-95)
 *   dg_rk3_step   replaces TakeRK3Step, the RKStep procedure pointer
 *                 (Solver/src/libs/timeintegrator/ExplicitMethods.f90:667-788,
 *                  TimeIntegrator.f90:215,292,809-813)
 *   dg_max_dt     replaces MaxTimeStep (Solver/src/libs/discretization/DGSEMClass.f90:870-1038)
 *   dg_residuals  replaces ComputeMaxResiduals (DGSEMClass.f90:770-868) and the NaN test of
 *                 checkForNan (ExplicitMethods.f90:1856-1908)
 *
 * All arrays crossing the boundary use the reference's own column-major layouts, element by
 * element in element order: Q(1:5,0:Nx,0:Ny,0:Nz) (StorageClass.f90:802), metric terms
 * jGradXi/Eta/Zeta(1:3,0:Nx,0:Ny,0:Nz), jacobian(0:Nx,0:Ny,0:Nz) (MappedGeometry.f90:24-35),
 * face geometry normal/t1/t2(1:3,0:Nf1,0:Nf2), jacobian(0:Nf1,0:Nf2) (MappedGeometry.f90:482-760).
 *
 * Every entry point returns an int status: DG_OK (0) or a negative DG_ERR_* code. No entry point
 * exits the process (the reference stops with `error stop`/exit(99); the caller maps the codes).
 * A context is not thread safe; use one context per host thread. Each context owns one CUDA stream.
 */
#ifndef HORSES3D_GB300_H
#define HORSES3D_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define DG_OK                0
#define DG_ERR_INVALID      -1   /* bad argument, inconsistent mesh description */
#define DG_ERR_UNSUPPORTED  -2   /* option outside the GPU path (caller keeps its CPU path) */
#define DG_ERR_CUDA         -3   /* a CUDA runtime call failed; dg_last_error() has the text */
#define DG_ERR_NAN          -4   /* NaN/Inf found in Q (checkForNan equivalent) */
#define DG_ERR_TIMEOUT      -5   /* a bounded device wait gave up */
#define DG_ERR_NOMEM        -6   /* device allocation failed */
#define DG_ERR_NODEVICE     -7   /* no CUDA device visible */
#define DG_ERR_IO           -8   /* mesh file could not be read */

/* ---- enumerations (values match the reference's keyword choices) ------------------------- */
enum { DG_NODES_GAUSS = 0, DG_NODES_GAUSS_LOBATTO = 1 };          /* "discretization nodes" */
enum { DG_INVISCID_STANDARD = 0, DG_INVISCID_SPLIT = 1 };          /* "inviscid discretization" */
enum { DG_RIEMANN_ROE = 0, DG_RIEMANN_LXF = 1,                    /* "riemann solver" */
       DG_RIEMANN_CENTRAL = 2, DG_RIEMANN_RUSANOV = 3,
       DG_RIEMANN_STD_ROE = 4, DG_RIEMANN_ROE_PIKE = 5,            /* "standard roe", "roe-pike" */
       DG_RIEMANN_LOW_DISS_ROE = 6,                                /* "low dissipation roe" */
       DG_RIEMANN_MATRIX_DISS = 7, DG_RIEMANN_VISCOUS_NS = 8,      /* "matrix dissipation", "viscous ns" */
       DG_RIEMANN_U_DISS = 9 };                                    /* "u-diss" */
enum { DG_AVG_STANDARD = 0, DG_AVG_PIROZZOLI = 1,                  /* "averaging" (the averaged */
       DG_AVG_DUCROS = 2, DG_AVG_MORINISHI = 3,                    /*  states of every solver but */
       DG_AVG_KENNEDY_GRUBER = 4,                                  /*  Roe and Rusanov, and the */
       DG_AVG_ENTROPY_CONSERVING = 5, DG_AVG_CHANDRASEKAR = 6 };   /*  split form's two-point fluxes) */
enum { DG_PRECISION_FP64 = 0, DG_PRECISION_MIXED = 1,             /* plain FP64 / FP32 flux form */
       DG_PRECISION_MIXED_TC = 2 };  /* mixed form with the gradient contractions and face traces on the
                                        tensor cores (tcgen05 TF32 split products in TMEM); uniform
                                        N = 5 on Gauss nodes, standard volume form, state gradients */
enum { DG_GRADVARS_STATE = 0, DG_GRADVARS_ENTROPY = 1,             /* "gradient variables" of BR1 */
       DG_GRADVARS_ENERGY = 2 };
enum { DG_SOURCE_NONE = 0,                                         /* UserDefinedSourceTermNS of */
       DG_SOURCE_MMS_CONVERGENCE = 1,                              /*  NavierStokes/Convergence */
       DG_SOURCE_MMS_LAMB_VECTOR = 2 };                            /*  NavierStokes/LambVector */
enum { DG_FIELD_Q = 0, DG_FIELD_QDOT = 1, DG_FIELD_G = 2,
       DG_FIELD_UX = 3, DG_FIELD_UY = 4, DG_FIELD_UZ = 5 };

/* Face-local element sides, numbered as the reference (HexElementConnectivityDefinitions.f90:69-77):
 * 1 FRONT (eta=-1), 2 BACK (eta=+1), 3 BOTTOM (zeta=-1), 4 RIGHT (xi=+1), 5 TOP (zeta=+1), 6 LEFT (xi=-1). */

/* Boundary conditions of non-periodic boundary zones (physics/common/*BC.f90, NAVIERSTOKES parts),
 * in the solver's dimensionless variables:
 *   NO_SLIP_WALL   NoSlipWallBC.f90:265-372   (wall velocity; adiabatic or isothermal)
 *   FREE_SLIP_WALL FreeSlipWallBC.f90:249-351 (adiabatic or isothermal)
 *   INFLOW         InflowBC.f90:363-414        (imposed rho, u, v, w, p; no turbulence intensity)
 *   OUTFLOW        OutflowBC.f90:226-304       (subsonic characteristic outflow at pressure p) */
enum { DG_BC_NO_SLIP_WALL = 1, DG_BC_FREE_SLIP_WALL = 2, DG_BC_INFLOW = 3, DG_BC_OUTFLOW = 4 };
typedef struct dg_boundary {
    int32_t type;                   /* DG_BC_* */
    int32_t isothermal;             /* walls: 0 adiabatic (reference default), 1 isothermal */
    double wall_temperature;        /* isothermal walls: T_wall / T_ref (reference default 1) */
    double wall_velocity[3];        /* no-slip walls (default 0) */
    double rho, u, v, w, p;         /* inflow state (defaults 1, the free stream at the AoA, 1/(gamma M^2)) */
    double pressure;                /* outflow pressure (default 1/(gamma M^2)) */
} dg_boundary;

/* Mesh description: geometry and connectivity as HexMesh holds them after ConstructGeometry.
 * Periodic faces count as interior faces (HexMesh.f90:519-736). A boundary face has a single
 * element: face_elem[2f+1] = -1, face_side[2f+1] = 0, face_rotation 0, face orders those of its
 * element side, its normal pointing out of the domain, and face_boundary[f] >= 0 naming its entry
 * of `boundaries`. */
typedef struct dg_mesh_desc {
    int32_t n_elements;
    int32_t node_type;              /* DG_NODES_* */
    const int32_t* order;           /* [3*K]  (Nx,Ny,Nz) of every element */
    const double* x;                /* [3*sum(P)] node coordinates x(1:3,i,j,k) */
    const double* ja_xi;            /* [3*sum(P)] jGradXi */
    const double* ja_eta;           /* [3*sum(P)] jGradEta */
    const double* ja_zeta;          /* [3*sum(P)] jGradZeta */
    const double* jacobian;         /* [sum(P)] */
    const double* inv_jacobian;     /* [sum(P)] */
    int32_t n_faces;
    const int32_t* face_elem;       /* [2*F] left, right element (0-based) */
    const int32_t* face_side;       /* [2*F] element side 1..6 of left, right */
    const int32_t* face_rotation;   /* [F]   0..7 (leftIndexes2Right, MeshTypes.f90:70-107) */
    const int32_t* face_nf;         /* [2*F] (Nf1,Nf2) face orders */
    const double* face_normal;      /* [3*sum(Pf)] unit normal, left -> right */
    const double* face_t1;          /* [3*sum(Pf)] */
    const double* face_t2;          /* [3*sum(Pf)] */
    const double* face_jacobian;    /* [sum(Pf)] surface Jacobian Jf */
    const int32_t* face_boundary;   /* [F] boundary condition of each boundary face, -1 for interior
                                       faces; NULL when every face is interior */
    int32_t n_boundaries;
    const dg_boundary* boundaries;  /* [n_boundaries] */
} dg_mesh_desc;

/* Physics constants (PhysicsStorage_NS.f90:186-429). gamma=1.4 (air) and Sutherland's law with
 * S=198.6*5/9 K, TRef=520*5/9 K are fixed as in the reference's defaults. */
typedef struct dg_physics {
    double mach;
    double reynolds;
    double prandtl;                 /* reference default 0.72 */
    int32_t navier_stokes;          /* 1: "NS" (BR1 viscous terms), 0: "Euler" (no gradients) */
} dg_physics;

typedef struct dg_options {
    int32_t inviscid;               /* DG_INVISCID_* (split form requires Gauss-Lobatto nodes) */
    int32_t riemann;                /* DG_RIEMANN_* */
    int32_t averaging;              /* DG_AVG_*  (LxF average and split-form two-point flux) */
    double lambda_stab;             /* LxF stabilisation factor, reference default 1.0 */
    int32_t precision;              /* DG_PRECISION_* */
    int32_t source;                 /* DG_SOURCE_* */
    int32_t gradient_variables;     /* DG_GRADVARS_* (SpatialDiscretization.f90:106-148) */
} dg_options;

typedef struct dg_ctx dg_ctx;

/* Library and device --------------------------------------------------------------------- */
const char* dg_version(void);
const char* dg_strerror(int code);
const char* dg_last_error(void);          /* text of the last failure on this thread */
int dg_device_count(int* count);

/* Context lifetime: copies the mesh description to device memory once (host pointers are not
 * retained). Replaces the one-time storage set-up of HexMesh (HexMesh.f90:5802). */
int dg_create(const dg_mesh_desc* mesh, const dg_physics* phys, const dg_options* opts, dg_ctx** out);
void dg_destroy(dg_ctx* ctx);

/* State transfer in the reference layout (Q(1:5,i,j,k) element after element). */
int dg_upload_state(dg_ctx* ctx, const double* q);
int dg_download(dg_ctx* ctx, int field, double* dst);
/* The mixed form carries the energy in FP32 relative to a constant reference, by default the mean
 * energy of each upload. Element partitions of one mesh must share one reference: set it after
 * dg_upload_state (e.g. to the mean over all partitions). Recomputes the face traces; no effect on
 * the plain form. Uniform-order contexts only. No reference counterpart (the reference is FP64). */
int dg_set_energy_reference(dg_ctx* ctx, double e_ref);
int64_t dg_ndof(const dg_ctx* ctx);

/* ComputeTimeDerivative: QDot = RHS(Q, t) (SpatialDiscretization.f90:227-685). */
int dg_rhs(dg_ctx* ctx, double t);

/* TakeRK3Step: three RHS evaluations at t + b_k dt and the low-storage updates
 * G = a_k G + QDot, Q = Q + c_k dt G (ExplicitMethods.f90:748-779). dt must be positive; for
 * CFL stepping call dg_max_dt first, as the reference's time loop does (TimeIntegrator.f90:748-754). */
int dg_rk3_step(dg_ctx* ctx, double t, double dt);

/* Keeps the lifted gradients U_x, U_y, U_z of the last RK stage of every step (dg_download of
 * DG_FIELD_UX..UZ after the step), which the reference's storage holds after TakeRK3Step and its
 * monitors read (enstrophy, VolumeIntegrals.f90:267). Off by default: it writes 15 values per node
 * per step. Navier-Stokes uniform-order contexts. */
int dg_keep_gradients(dg_ctx* ctx, int on);

/* n RK3 steps from t0 entirely on the device, captured once in a CUDA graph and replayed: no host
 * synchronisation between steps. dt > 0: fixed step. dt <= 0: every step takes the MaxTimeStep
 * value for (cfl, dcfl), computed and applied on the device. t_end (may be NULL) receives the final
 * time (this synchronises). */
int dg_run_steps(dg_ctx* ctx, int n, double t0, double dt, double cfl, double dcfl, double* t_end);

/* IntegrateInTime's explicit loop on the device (TimeIntegrator.f90:737-890 without output): n steps
 * from t0, each MaxTimeStep (when dt <= 0, with cfl/dcfl) + TakeRK3Step + t += dt +
 * ComputeMaxResiduals / checkForNan, replayed from one CUDA graph with a single host synchronization at
 * the end. residuals (optional) receives [n][n_cases][5] maximum |QDot| after each step; *nan_step the
 * first step (1-based) whose state held a NaN/Inf, then DG_ERR_NAN is returned (the steps after it
 * ran on the non-finite state; the reference would have stopped there). */
int dg_integrate(dg_ctx* ctx, int n, double t0, double dt, double cfl, double dcfl, double* t_end,
                 double* residuals, int* nan_step);

/* dg_run_steps timed with CUDA events recorded on the context's stream around the graph
 * launches; *ms receives the elapsed device time. Measurement helper, no reference counterpart. */
int dg_time_steps(dg_ctx* ctx, int n, double t0, double dt, double cfl, double dcfl, double* ms);

/* Average device time (ms) of each kernel launched alone reps times on the context's stream:
 * ms[0] volume (gradient, BR1 lifting, volume integral), ms[1] face flux, ms[2] surface integral +
 * RK update + traces, ms[3] traces alone, ms[4] unused (0). Advances Q by reps RK stage-1 updates
 * of size dt. Measurement helper, no reference counterpart. */
int dg_kernel_times(dg_ctx* ctx, int reps, double t0, double dt, double ms[5]);

/* FP64 fused multiply-add throughput of the current device in TFLOP/s (2 flops per FMA), from
 * independent FMA chains over a grid that fills every SM, timed with CUDA events: the denominator
 * of the plain FP64 form's compute roofline. Measurement helper, no reference counterpart. */
int dg_measure_fp64_peak(double* tflops);

/* Self-test of the tensor-core building blocks: C (128 x 16) = A (128 x 8) * B (16 x 8)^T, host
 * row-major FP32 arrays, computed by tcgen05 TF32 MMAs in TMEM (split = 0: one TF32 product;
 * split = 1: the three-term TF32 split product, about FP32 accurate). Test helper, no reference
 * counterpart. */
int dg_tc_selftest(const float* a, const float* b, float* c, int split);

/* MaxTimeStep (DGSEMClass.f90:870-1038) on the device. */
int dg_max_dt(dg_ctx* ctx, double cfl, double dcfl, double* dt);

/* MaxTimeStep without any device allocation, for callers that cannot call cudaMalloc (a host that
 * owns all device memory through its own pool, or code running after an allocation freeze). No
 * counterpart in the reference. The caller passes device pointers in the reference layouts:
 * q (5*ndof), ja_xi/ja_eta/ja_zeta (3*ndof), jacobian (ndof), for uniform order `order`. The only
 * scratch is a fixed 128 KiB file-scope device array that every GPU loading the library keeps until
 * exit; it bounds ndof to dg_max_dt_noalloc_max_dof() (67,108,864) and larger sizes are rejected
 * with DG_ERR_INVALID. The first call on a device looks up that array's address in the device's
 * current context and keeps it; after a cudaDeviceReset of that device the kept address is stale, so
 * do not call this function on a device that the process has reset. Every call reuses the array, so
 * calls that overlap on the GPU (other streams or threads) race; each call overwrites the entries it
 * reads. stream may be NULL (default stream); the call synchronises it and writes dt to host memory,
 * so it cannot run while the stream is being captured into a CUDA graph (DG_ERR_UNSUPPORTED). A
 * CUDA error already pending when the call starts is returned as DG_ERR_CUDA without launching. */
int dg_max_dt_noalloc(const double* q, const double* ja_xi, const double* ja_eta, const double* ja_zeta,
                      const double* jacobian, int64_t ndof, int order, int node_type, const dg_physics* phys,
                      double cfl, double dcfl, void* stream, double* dt);
int64_t dg_max_dt_noalloc_max_dof(void);

/* ComputeMaxResiduals: max|QDot| per conserved variable; *nan_found = 1 if Q holds NaN/Inf. */
int dg_residuals(dg_ctx* ctx, double maxres[5], int* nan_found);

/* Element partitions (multi-GPU domain decomposition, one partition per GPU; the reference's MPI
 * path: MPI_Face.f90:203-383, HexMesh_UpdateMPIFacesSolution/Gradients in HexMesh.f90:1199-1730,
 * the dt and residual reductions of DGSEMClass.f90:1019-1021 and :770-868).
 *
 * dg_create_partition: `mesh` describes the partition's own elements (n_elements, with their nodes
 * and metric terms) and every face that touches them. A face to a remote element names it as
 * n_elements + g, g in 0..n_ghost-1 (`order` holds 3*(n_elements + n_ghost) entries; one isotropic
 * order throughout), keeps the global face's left/right sides, rotation and geometry, and must have
 * one of the partition's own elements. Each ghost element owns six face slots (slot = 6*element +
 * side - 1) that the halo exchange fills; it has no nodes. */
int dg_create_partition(const dg_mesh_desc* mesh, int32_t n_ghost, const dg_physics* phys, const dg_options* opts,
                        dg_ctx** out);
/* Registers the slots packed for the neighbours (own slots, 0 .. 6*n_elements-1) and the ghost
 * slots filled from them (6*n_elements .. 6*(n_elements+n_ghost)-1), in the order both sides agree
 * on (e.g. neighbour by neighbour, faces in global order). */
int dg_halo_set_slots(dg_ctx* ctx, int32_t n_send, const int32_t* send_slots, int32_t n_recv, const int32_t* recv_slots);
/* Bytes of one slot's payload: P^2 points x 5 values of the working precision (8 bytes plain, 4 mixed). */
int64_t dg_halo_slot_bytes(const dg_ctx* ctx);
/* DG_HALO_Q_TRACES: the Q traces of the current state, exchanged before the volume phase.
 * DG_HALO_VISCOUS_FLUX: each side's viscous normal flux Fv(Q, grad U).n, exchanged before the
 * surface phase (Navier-Stokes only). dst/src are device buffers of n_send/n_recv slot payloads;
 * both calls return when the data is in place. */
enum { DG_HALO_Q_TRACES = 0, DG_HALO_VISCOUS_FLUX = 1 };
int dg_halo_pack(dg_ctx* ctx, int field, void* dst);
int dg_halo_unpack(dg_ctx* ctx, int field, const void* src);
/* One half of an RK stage on a partition: phase 0 the volume kernel (gradients, BR1 lifting, the
 * sides' viscous normal fluxes, volume integral), phase 1 the face fluxes and the surface integral
 * with the low-storage update of RK stage `stage` (0..2, at time t + b_k dt, then the Q traces of the
 * new state) or, with stage -1, the right-hand side alone at time t (QDot and the lifted gradients
 * kept). A step is, for k = 0..2: exchange Q traces, phase 0, exchange viscous fluxes (NS), phase 1;
 * dt and residuals are reduced over the partitions by the caller (MIN, MAX). */
int dg_partition_stage(dg_ctx* ctx, int stage, int phase, double t, double dt);

/* Block until all work queued on the context's stream is done. */
int dg_synchronize(dg_ctx* ctx);

/* Batches of independent cases in one context (no reference counterpart: the reference runs one
 * case per process). Every case has its own mesh (any orders), physics constants, time and dt;
 * the options and the node type are shared. All cases are advanced by the same kernel launches
 * (elements bucketed by order triple), each with its own dt. The state arrays of the single-case
 * entry points (dg_upload_state, dg_download) hold the cases one after the other, case k starting
 * at node dg_case_offset(ctx, k). On a batch, dg_rk3_step/dg_run_steps give every case the same
 * t and dt, dg_max_dt returns the smallest case dt (each case keeps its own on the device) and
 * dg_residuals the maximum over the cases. dg_create itself routes a mesh with anisotropic or
 * element-varying orders to this path as a batch of one. */
int dg_create_batch(int n_cases, const dg_mesh_desc* meshes, const dg_physics* phys, const dg_options* opts,
                    dg_ctx** out);
int dg_batch_size(const dg_ctx* ctx);
int64_t dg_case_offset(const dg_ctx* ctx, int k);                    /* k in 0..n_cases; -1 if out of range */
int dg_batch_set_clock(dg_ctx* ctx, const double* t, const double* dt);   /* [n_cases] each */
int dg_batch_get_clock(dg_ctx* ctx, double* t, double* dt);
/* MaxTimeStep of every case into dt[n_cases]; the values also become the cases' device dt. */
int dg_batch_max_dt(dg_ctx* ctx, double cfl, double dcfl, double* dt);
/* Per-case residuals maxres[5*n_cases] and NaN flags nan_found[n_cases] (may be NULL). */
int dg_batch_residuals(dg_ctx* ctx, double* maxres, int* nan_found);
/* Autotuner of the variable-order / batch kernels: for every order triple of the context, times the
 * volume and update kernels with several elements-per-CTA sizes (reps launches each, best of three)
 * and keeps the fastest per DOF. The choice is cached per (order triple, precision, equations, node
 * type) for the process, so later contexts with those triples start tuned; with the environment
 * variable HORSES3D_GB300_TUNE_FILE set, the table is read from and written to that file. The
 * state (Q, G, QDot) is restored afterwards. A no-op (DG_OK) on uniform-order contexts. */
int dg_autotune(dg_ctx* ctx, int reps);
/* Failure-path test hook. DG_FAULT_TMA_WAIT makes the update kernels of the bulk-copy (TMA) path
 * (uniform order N=5) expect 16 bytes that no copy delivers, so their bounded mbarrier waits run
 * out (after about two seconds): every CTA records the failure and leaves, and the entry point
 * returns DG_ERR_TIMEOUT; the state is then invalid and must be uploaded again. DG_FAULT_NONE
 * restores normal operation. No copy is left in flight by the injected fault. DG_ERR_UNSUPPORTED on
 * contexts without such waits. */
enum { DG_FAULT_NONE = 0, DG_FAULT_TMA_WAIT = 1 };
int dg_inject_fault(dg_ctx* ctx, int kind);
/* n RK3 steps of every case from its device clock (CUDA-graph replay). cfl > 0: every step takes
 * each case's MaxTimeStep(cfl, dcfl); otherwise each case's current dt. ms (may be NULL) receives
 * the device time measured with events on the context's stream. */
int dg_batch_run_steps(dg_ctx* ctx, int n, double cfl, double dcfl, double* ms);
/* dg_integrate for a batch from each case's own clock (dg_batch_set_clock): MaxTimeStep per case
 * each step when cfl > 0, else each case's dt; residuals [n][n_cases][5]. */
int dg_batch_integrate(dg_ctx* ctx, int n, double cfl, double dcfl, double* residuals, int* nan_step);

/* HORSES3D solution files (.hsol; io/SolutionFile.f90, HexMesh_SaveSolution/LoadSolution in
 * HexMesh.f90:3376-3555,4708-). Host functions, no device needed. The gradient array of a type-3
 * file holds, element after element, U_x, U_y, U_z (5 values per node each, reference layout). */
typedef struct h3d_solution_header {
    char name[128];          /* the name given at creation (not NUL-terminated when 128 long) */
    int32_t file_type;       /* 2 solution, 3 solution and gradients (SolutionFile.f90:61-70) */
    int32_t node_type;       /* 1 Gauss, 2 Gauss-Lobatto (the reference's numbering) */
    int32_t n_elements;
    int32_t iteration;
    double time;
    double refs[6];          /* gamma, R, V_ref, rho_ref, T_ref, Mach */
} h3d_solution_header;
int h3d_read_solution_header(const char* path, h3d_solution_header* header);
/* Reads Q (5 per node, element order) and, when gradients is not NULL, the gradients of a type-3
 * file; every element record must have the orders given in orders[3*n_elements]. */
int h3d_read_solution(const char* path, int32_t n_elements, const int32_t* orders, double* q, double* gradients);
/* Writes a type-2 file (gradients NULL) or a type-3 file (header->file_type must agree). */
int h3d_write_solution(const char* path, const h3d_solution_header* header, const int32_t* orders, const double* q,
                       const double* gradients);

/* Saves case case_index of a context (0 for a single case) as a solution file written from the
 * device state, with iteration and time in the header and the reference values of the case's Mach
 * number (PhysicsStorage_NS.f90:290-310: T_ref = 520*5/9 K, p_ref = 101325 Pa, R = 287.15). With
 * with_gradients (Navier-Stokes only) the lifted gradients of the current state are computed (one
 * right-hand side at `time`) and written too (file type 3). */
int dg_save_solution(dg_ctx* ctx, int case_index, const char* path, int iteration, double time, int with_gradients);
/* Restart: loads Q of case case_index from a solution file (type 2 or 3, matching node type and
 * element orders), uploads it and returns the file's iteration and time (either may be NULL). */
int dg_load_solution(dg_ctx* ctx, int case_index, const char* path, int* iteration, double* time);

/* Host-side mesh builder (HexMesh construction: Read_SpecMesh.f90:36-342, HexMesh.f90:356-736,
 * 2677-2990, MappedGeometry.f90:64-760). Produces a dg_mesh_desc whose arrays live in the mesh. */
typedef struct h3d_mesh h3d_mesh;

/* periodic: comma separated "plus:minus" boundary-name pairs (case-insensitive), e.g.
 * "front:back,bottom:top,left:right". orders: [3*K] per-element orders or NULL for uniform
 * (uniform_n used in all three directions). */
int h3d_mesh_read_specmesh(const char* path, int node_type, int uniform_n, const int32_t* orders,
                           const char* periodic, h3d_mesh** out);
/* Periodic box [x0,x1]x[y0,y1]x[z0,z1] of nx*ny*nz hexahedra, optionally warped by
 * x_i += warp*sin(x)sin(y)sin(z) with curved faces given as Chebyshev-Lobatto patches of order
 * patch_order (patch_order < 2 and warp == 0 gives straight-sided hex8 elements). */
int h3d_mesh_box(int nx, int ny, int nz, const double lo[3], const double hi[3], double warp,
                 int patch_order, int node_type, int uniform_n, const int32_t* orders, h3d_mesh** out);
/* The same box with a chosen periodic-pair list ("left:right,..." over the zone names left/right
 * (x), front/back (y), bottom/top (z)); the other zones become boundary zones. */
int h3d_mesh_box_zones(int nx, int ny, int nz, const double lo[3], const double hi[3], double warp,
                       int patch_order, int node_type, int uniform_n, const int32_t* orders,
                       const char* periodic, h3d_mesh** out);
/* Fills out with the mesh's arrays. Boundary faces get face_boundary = the index of their zone
 * (h3d_mesh_zone_name) and n_boundaries = the number of zones; `boundaries` is left NULL for the
 * caller to point at one dg_boundary per zone. */
int h3d_mesh_describe(const h3d_mesh* mesh, dg_mesh_desc* out);
/* Non-periodic boundary zones of the mesh (SpecMesh boundary names, lower case). */
int h3d_mesh_zone_count(const h3d_mesh* mesh);
const char* h3d_mesh_zone_name(const h3d_mesh* mesh, int zone);
/* Total quadrature volume sum_e sum_ijk w_i w_j w_k J (MappedGeometry.f90:132-135). */
double h3d_mesh_volume(const h3d_mesh* mesh);
void h3d_mesh_free(h3d_mesh* mesh);

/* Nodal storage of order n (NodalStorageClass.f90:170-338): fills x,w [n+1] and D [(n+1)^2,
 * row-major D(i,j)]. Any pointer may be NULL. */
int h3d_nodal_storage(int node_type, int n, double* x, double* w, double* d);

#ifdef __cplusplus
}
#endif

#endif /* HORSES3D_GB300_H */
