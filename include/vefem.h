/*
 * vefem.h -- C ABI of the GB300 (sm_103a) element-assembly library for the
 * viscoelastic flow-around-a-cylinder solver.
 *
 * It replaces the reference's bulk assembly call
 *     call setEquationsBulk(Problem, FE, Mesh, Boundary, GaussInt, Sol, &
 *                           basis_p, Flag_NR, Elem, LS)
 * (Equations_mod.F90:21-55, called from assemblePetscObjects,
 * Newton_Raphson_mod.F90:332) and, optionally, the outlet open-boundary edge
 * terms (setEquationsEdge, Equations_mod.F90:317-554, called at
 * Newton_Raphson_mod.F90:349).  Like VecSetValues/MatSetValues with
 * ADD_VALUES (Storage_mod.F90:10-115) it ADDS the element residuals into the
 * global residual b and the element Jacobians into the values array of a
 * frozen AIJ (CSR) pattern, one element after another in element order, so
 * the global sums are bit-for-bit those of the reference's sequential loop.
 *
 * All arrays use the reference's own (Fortran column-major) layouts, so a
 * Fortran host passes its arrays through iso_c_binding without copies:
 *   conn  : Mesh%Connectivity(Nel, 9)   -> conn[inod*nel + iel], 1-based ids
 *   xyz   : Mesh%Xi_Mesh(Nnodes, 3)     -> xyz[j*nnodes + node]
 *   TL    : Sol%TL(Nnodes, Neq=6)       -> TL[ieq*nnodes + node]
 *           field order Ux, Uy, P, Txx(Sxx), Txy(Sxy), Tyy(Syy)
 *   EU    : Sol%EU(Nex)                 (Nex = 1: the arclength parameter ArN)
 *   b     : LS%b_f, length N = Nnodes*6 + Nex, row (gnode-1)*6 + ieq-1
 *   vals  : the AIJ values array of LS%A_f (MatSeqAIJGetArray), CSR order
 *
 * Errors: every entry point returns an int status (0 = OK), mirroring
 * PETSc's ierr; the library never exits.  vefem_last_error() gives text.
 * One context is used by one host thread at a time.
 */
#ifndef VEFEM_H
#define VEFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VEFEM_ABI_VERSION 1

/* status codes */
#define VEFEM_OK 0
#define VEFEM_ERR_ARG 1          /* invalid argument or size */
#define VEFEM_ERR_PATTERN 2      /* CSR pattern lacks an element entry or is not node-blocked */
#define VEFEM_ERR_CUDA 3         /* CUDA runtime error (text in vefem_last_error) */
#define VEFEM_ERR_NOMEM 4        /* host or device allocation failed */
#define VEFEM_ERR_UNSUPPORTED 5  /* option not available in this build */
#define VEFEM_ERR_SINGULAR 6     /* vefem_frontal_factor: a pivot below the tolerance */

/* constitutive models, in the order of setConEQ_T / setConEQ_SQRT
 * (Constitutive_Models_mod.F90:31-49, Constitutive_Models_SQRT_mod.F90:66-84) */
#define VEFEM_MODEL_L_PTT 0      /* Oldroyd-B is L-PTT with VeN = 0 */
#define VEFEM_MODEL_M_L_PTT 1
#define VEFEM_MODEL_E_PTT 2
#define VEFEM_MODEL_M_E_PTT 3
#define VEFEM_MODEL_FENE_CR 4
#define VEFEM_MODEL_FENE_P 5
#define VEFEM_MODEL_GIESEKUS 6

/* stress formulation, Parameters_mod.F90:122 (Stress_Reform) */
#define VEFEM_FORM_T 0           /* polymer stress T */
#define VEFEM_FORM_SQRT 1        /* square-root conformation S, c = S.S */

/* vefem_assemble flags */
#define VEFEM_RESIDUAL 0x1       /* add the element residuals into b ('MNR' and 'NRP') */
#define VEFEM_JAC_FD64 0x2       /* add the FP64 forward-difference Jacobian ('NRP'),
                                    the reference algorithm of storeBulk, bit-exact */
#define VEFEM_JAC_EXACT64 0x4    /* add the exact (linearised) Jacobian in FP64: forward-mode
                                    derivative of the same physics, no FD truncation error */
#define VEFEM_JAC_EXACT32 0x8    /* the exact Jacobian in FP32 into a float AIJ values array:
                                    the inexact-Newton precision form (residual stays FP64) */
#define VEFEM_ZERO_FIRST 0x100   /* zero b (and vals when a Jacobian is requested) before
                                    adding, like initializeLSObjects (Petsc_mod.F90:747-763) */
#define VEFEM_OUTLET_EDGES 0x200 /* also add the outlet open-BC edge terms (openBC,
                                    Residuals_mod.F90:599-624) of the mesh's outlet edges */
#define VEFEM_TIMING 0x1000      /* record per-kernel CUDA-event times (vefem_last_timing) */

/* Run-time form of the reference's compile-time physics parameters
 * (Parameters_mod.F90:98-122).  With nex = 1 (arclength continuation in Wi)
 * the Weissenberg number at every Gauss point is Wi0 * EU[0]
 * (setContinuationParameter, Element_Calculations_mod.F90:577-601);
 * with nex = 0 it is WiN.  dt is huge(1d0) for steady runs
 * (Physical_mod.F90:345); fd_eps is the absolute FD step (1e-8,
 * perturbVariableReal, Tools_mod.F90:831-840). */
typedef struct vefem_params {
    int32_t model;
    int32_t form;
    int32_t nex;                 /* 0 or 1 */
    int32_t device;              /* CUDA device ordinal the context runs on */
    double ReN, WiN, BvN, VeN, DfN, Wi0, dt, fd_eps;
} vefem_params;

typedef struct vefem_mesh {
    int32_t nnodes;
    int32_t nel;
    const int32_t *conn;         /* [9 * nel], conn[inod*nel + iel], 1-based node ids */
    const double *xyz;           /* [3 * nnodes], xyz[j*nnodes + node] (z unused in 2-D) */
    int32_t n_outlet_edges;      /* outlet edges for VEFEM_OUTLET_EDGES (may be 0) */
    const int32_t *outlet_edge_elem;  /* [n] 0-based element of each edge (edge_elements_rank - 1) */
    const int32_t *outlet_edge_id;    /* [n] local edge id 1..4: eta=-1, xi=+1, eta=+1, xi=-1 */
} vefem_mesh;

typedef struct vefem_csr {
    int64_t n;                   /* rows = cols = nnodes*6 + nex */
    const int64_t *rowptr;       /* [n + 1], 0-based */
    const int32_t *colind;       /* [rowptr[n]], sorted within each row */
} vefem_csr;

typedef struct vefem_ctx vefem_ctx;

/* Build the device-side tables for one mesh and one frozen AIJ pattern:
 * gather map, per-node residual contributor lists, per node-pair CSR block
 * offsets and contributor lists (the deterministic element-ordered scatter),
 * and the Gauss/basis tables.  Replaces the preallocation the reference does
 * with zero element blocks (preAllocatePetsc, Petsc_mod.F90:629-743): the
 * pattern must contain every element block, and, when nex = 1, the last
 * column in every node row. */
int vefem_create(const vefem_mesh *mesh, const vefem_csr *pattern, const vefem_params *params,
                 vefem_ctx **out);

/* Change the physics parameters (model, form, Wi, beta, ...); nex must not change. */
int vefem_set_params(vefem_ctx *ctx, const vefem_params *params);

/* One bulk assembly: setEquationsBulk with Flag_NR = 'MNR' (VEFEM_RESIDUAL)
 * or 'NRP' (VEFEM_RESIDUAL | one Jacobian flag: VEFEM_JAC_FD64 is the
 * reference's algorithm; VEFEM_JAC_EXACT64 / VEFEM_JAC_EXACT32 the exact
 * derivative in FP64 / FP32).
 * on_device = 0: TL, EU, b, vals are host pointers (copied in and out;
 *                pinned memory gives full link speed);
 * on_device = 1: they are device pointers (CUDA unified addressing).
 * vals is double[nnz] (float[nnz] with VEFEM_JAC_EXACT32) and may be NULL
 * when no Jacobian is requested.  Outlet edges (VEFEM_OUTLET_EDGES) always
 * use the FD Jacobian.  The call returns when the results are in b and vals. */
int vefem_assemble(vefem_ctx *ctx, const double *TL, const double *EU, int flags, double *b,
                   void *vals, int on_device);

/* Dirichlet rows after assembly, as applyDirichletBC and
 * applyDirichletBCFullyDeveloped do (Dirichlet_mod.F90:104-192):
 * b[row] = TL(node, eq) - value (INSERT) for every listed row, and, when
 * flags holds a Jacobian flag, the row's AIJ entries are zeroed and its
 * diagonal set to 1 (MatZeroRows with diag = 1).  rows are 0-based global
 * rows (node*6 + eq) of node unknowns, without duplicates; values the
 * prescribed values.  flags: VEFEM_RESIDUAL (update b) and at most one
 * Jacobian flag (VEFEM_JAC_EXACT32 means vals is float[nnz]).
 * on_device = 1: rows, values, TL, b, vals are device pointers; 0: host. */
int vefem_apply_dirichlet(vefem_ctx *ctx, int nrows, const int64_t *rows, const double *values,
                          const double *TL, double *b, void *vals, int flags, int on_device);

/* Per-kernel times (milliseconds, CUDA events on the context's stream) of the
 * last vefem_assemble called with VEFEM_TIMING:
 * t[0] element kernel, t[1] residual scatter, t[2] Jacobian scatter,
 * t[3] edge kernel + scatter, t[4] host<->device copies.  n = entries wanted. */
int vefem_last_timing(const vefem_ctx *ctx, float *t, int n);

/* Number of kernels the library launched in the last vefem_assemble. */
int vefem_last_launch_count(const vefem_ctx *ctx);

/* The CUDA stream the context launches on (cudaStream_t as void*). */
void *vefem_stream(const vefem_ctx *ctx);

int vefem_destroy(vefem_ctx *ctx);

/* Text of the last error of ctx (or of the last failed vefem_create when ctx is NULL). */
const char *vefem_last_error(const vefem_ctx *ctx);

/* Host helper: the AIJ pattern preAllocatePetsc freezes (Petsc_mod.F90:629-743)
 * for a mesh, for hosts without PETSc.  Call once with rowptr/colind NULL to
 * get n and nnz, then again with arrays of those sizes. */
int vefem_build_pattern(const vefem_mesh *mesh, int nex, int64_t *n, int64_t *nnz,
                        int64_t *rowptr, int32_t *colind);

/* Algorithmic FP64 operation count per element of the element kernel that
 * vefem_assemble runs for these flags (VEFEM_JAC_FD64 set: residual + FD
 * Jacobian, 56 residual evaluations; else the residual alone), obtained by
 * running the kernels' own physics source with an op-counting scalar.
 * out[0] = total (+, -, *, /, sqrt, exp count one each), out[1..5] = the
 * add/sub, mul, div, sqrt and exp parts.  Used for roofline reporting. */
int vefem_algorithmic_ops(const vefem_params *params, int flags, double *out);

/* Residual-only bulk assembly ('MNR') that allocates no device memory.  No
 * counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc when they assemble (device memory owned by another allocator or
 * pool, allocation-free sections, no long-lived library context).
 * All pointers are device pointers: conn [9*nel] (Connectivity(Nel,9),
 * 1-based), xyz [3*nnodes], TL [6*nnodes], EU [nex], b [nnodes*6 + nex];
 * the residual is ADDED into b (rows of the arclength unknown untouched),
 * bit-identical to vefem_assemble(VEFEM_RESIDUAL).  stream: a cudaStream_t
 * (NULL = default stream); the call synchronises that stream (it reads a
 * device-side error flag) before it returns, and it leaves the caller's
 * current device as it found it.
 * Scratch is one static device array of about 17.7 MB that every GPU loading
 * the library holds until exit.  Limits, each rejected with VEFEM_ERR_ARG:
 * at most 32768 elements and 294912 nodes (checked before anything runs);
 * at most 32 elements sharing one node, and connectivity ids in 1..nnodes
 * (checked on the device before anything is added: b is left unchanged).
 * The first call on a device looks up that array's address and uploads the
 * Gauss tables: make it before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race. */
int vefem_assemble_residual_noalloc(const vefem_params *params, int nnodes, int nel,
                                    const int32_t *conn, const double *xyz, const double *TL,
                                    const double *EU, double *b, void *stream);

int vefem_abi_version(void);

/* ---- Linear solver: panel-frontal elimination on the device ----------------
 * The numeric phases of the Newton drivers' direct solve, in place of the
 * MUMPS factorisation and solve behind KSPSolve (Petsc_mod.F90:850; the
 * bordered matrix of the arclength continuation, Extra_Equations_mod.F90:
 * 698-829, included).  The symbolic phase is the caller's (the package's
 * frontal.py): npan frontal matrices, panel q's n[q] x n[q] matrix row-major at
 * buf + off[q], its p[q] pivots first and its front after them; idx
 * [idx_off[q] .. idx_off[q+1]) the global unknown of every row/column of panel
 * q (device, int64); ext [ext_off[q] ..) the position in panel q+1 of each
 * front unknown of panel q (device, int32).  Every unknown is a pivot of
 * exactly one panel (the p[q] sum to N).  The device arrays are the caller's
 * and must outlive the handle; create reads idx once, synchronously, to set up
 * the solve's elimination order (N and the entries of idx below 2^31).
 * vefem_frontal_factor: buf holds the assembled original entries of every
 * panel (zeros elsewhere); the elimination (blocked Gauss-Jordan without
 * pivoting, with the Schur complement of each panel added into the next one)
 * overwrites it with the factors.  Returns VEFEM_ERR_SINGULAR when a pivot is
 * at most tol times the largest entry of its 16 x 16 pivot block (the caller
 * then factorises with pivoting); min_pivot (may be NULL) receives the
 * smallest such ratio.  Synchronises the stream.
 * vefem_frontal_solve: x = A^-1 b with the factors in buf; b and x are device
 * vectors of N doubles (b is not modified).  The sweeps (two launches per
 * panel, chained by programmatic dependent launch where the driver accepts it)
 * are captured once per buf into a CUDA graph and replayed; asynchronous on
 * the stream.
 * vefem_frontal_solve_path: how the last solve's launches were chained (1
 * programmatic dependent launch, 2 plain stream order; -1 no solve yet).
 * stream: a cudaStream_t (NULL = default stream). */
typedef struct vefem_frontal vefem_frontal;

int vefem_frontal_create(int device, int npan, const int64_t *off, const int32_t *n,
                         const int32_t *p, const int32_t *ext, const int64_t *ext_off,
                         const int64_t *idx, const int64_t *idx_off, int64_t N,
                         vefem_frontal **out);
int vefem_frontal_factor(vefem_frontal *f, double *buf, void *stream, double tol,
                         double *min_pivot);
int vefem_frontal_solve(vefem_frontal *f, const double *buf, const double *b, double *x,
                        void *stream);
void vefem_frontal_destroy(vefem_frontal *f);
const char *vefem_frontal_last_error(const vefem_frontal *f);
int vefem_frontal_solve_path(const vefem_frontal *f);

/* ---- Linear stability: batched A/B assembly --------------------------------
 * setEquationsBulkStability (Stability/Equations_Stability_mod.F90:20-226):
 * the matrices of the generalised eigenproblem A x = lambda B x for
 * spanwise-periodic 3-D perturbations of the steady 2-D state, 10 unknowns
 * per node (Ux, Uy, Uz, P, Txx, Txy, Tyy, Txz, Tyz, Tzz), node-major rows.
 * TLb [10][nnodes] is the base embedded as updateStabilityArrays does
 * (Continuation_Stability_mod.F90:592-633: [Ux, Uy, 0, P, Txx, Txy, Tyy, 0, 0, 0]);
 * Wi is params.WiN.  A[k] receives A at wavenumber kw[k] (k = 0..nk-1) and B
 * the k-independent B, ADD semantics, on the pattern vefem_stability_pattern
 * returns (query sizes with rowptr = colind = NULL first).  T form and the
 * L-PTT, m-L-PTT, e-PTT, m-e-PTT and Giesekus models; Dirichlet rows are the
 * caller's (applyDirichletBCStability: A row -> unit row, B row -> 0).
 * The reference comments out the z-derivatives of the perturbation
 * (Element_Calculations_Stability_mod.F90:52-79); they are included unless
 * VEFEM_STAB_AS_WRITTEN is given. */
#define VEFEM_STAB_AS_WRITTEN 0x2000

int vefem_stability_pattern(vefem_ctx *ctx, int64_t *n, int64_t *nnz, int64_t *rowptr,
                            int32_t *colind);
int vefem_stability_assemble(vefem_ctx *ctx, const double *TLb, int nk, const double *kw,
                             int flags, double *const *A, double *B, int on_device);

/* ---- Batched form ---------------------------------------------------------
 * Many independent instances (Weissenberg points, meshes of uneven size)
 * assembled by one persistent launch per kernel, replayed as a CUDA graph.
 * Each instance is what one vefem_create would take; the batched call is
 * setEquationsBulk (Equations_mod.F90:21-55) for every instance at once,
 * with the same ADD semantics and bit-identical results to one
 * vefem_assemble per instance.  All instances must share the device, the
 * conformation form and the zero/non-zero pattern of ReN and DfN.
 * Flags: VEFEM_RESIDUAL, VEFEM_JAC_EXACT32 or VEFEM_JAC_EXACT64,
 * VEFEM_ZERO_FIRST, VEFEM_TIMING (VEFEM_JAC_FD64 and VEFEM_OUTLET_EDGES are
 * VEFEM_ERR_UNSUPPORTED here: the outlet edges are the separate reference
 * call setEquationsEdge).  Arrays of pointers, one per instance; vals are
 * double for EXACT64 and float for EXACT32.  With on_device = 1 the first
 * call for a flag set captures a CUDA graph, later calls replay it. */
typedef struct vefem_batch vefem_batch;

int vefem_batch_create(int ninst, const vefem_mesh *meshes, const vefem_csr *patterns,
                       const vefem_params *params, vefem_batch **out);
int vefem_batch_set_params(vefem_batch *bt, int inst, const vefem_params *params);
int vefem_assemble_batched(vefem_batch *bt, const double *const *TL, const double *const *EU,
                           int flags, double *const *b, void *const *vals, int on_device);
/* Element-batch tile per mesh-size class (class c: nel in [1000*2^c, 1000*2^(c+1)),
 * c clamped to 0..VEFEM_BATCH_CLASSES-1).  vefem_batch_autotune times every
 * candidate tile of every class present on the live GPU (reps launches each,
 * device-resident buffers of its own) and keeps the fastest; tiles_out
 * (may be NULL) receives the chosen tiles. */
#define VEFEM_BATCH_CLASSES 6
int vefem_batch_autotune(vefem_batch *bt, int flags, int reps, int *tiles_out);
int vefem_batch_set_tiles(vefem_batch *bt, const int *tiles);
/* out[0] instances, out[1] elements, out[2] work items of the Jacobian kernel,
 * out[3] its persistent grid, out[4] kernels launched by the last call,
 * out[5] graph replays so far */
int vefem_batch_info(const vefem_batch *bt, int64_t out[6]);
/* with VEFEM_TIMING: ms[0] element kernels, ms[1] scatter, ms[2] copies and zeroing */
int vefem_batch_last_timing(const vefem_batch *bt, float ms[3]);
int vefem_batch_destroy(vefem_batch *bt);
const char *vefem_batch_last_error(const vefem_batch *bt);

/* ---- Learned continuation predictor: network kernels ---------------------
 * No counterpart in the reference (its arclength predictor is the tangent
 * step of updateSolutionArclength, Continuation_Arclength_mod.F90:339-379).
 * A multilayer perceptron in -> width -> ... -> width -> out with
 * hidden_layers GELU layers (erf form) and a linear output, BF16 weights
 * (FP32 master copies) with FP32 accumulation, trained by full-batch Adam
 * (beta1 0.9, beta2 0.999, eps 1e-8) on the mean squared error.  Host
 * pointers throughout; every call returns after its work has finished.
 * Parameters are one FP32 array: for each layer W[out][in] then b[out]. */
typedef struct vefem_mlp vefem_mlp;

int vefem_mlp_create(int in_dim, int width, int out_dim, int hidden_layers, uint64_t seed,
                     int device, vefem_mlp **out);
int64_t vefem_mlp_num_params(const vefem_mlp *m);
int vefem_mlp_set_params(vefem_mlp *m, const float *params, int64_t n);
int vefem_mlp_get_params(const vefem_mlp *m, float *params, int64_t n);
/* Y[n][out] = net(X[n][in]) */
int vefem_mlp_forward(vefem_mlp *m, const float *X, int n, float *Y);
/* loss = mean((net(X) - T)^2) and its gradient in the parameter layout */
int vefem_mlp_loss_grad(vefem_mlp *m, const float *X, const float *T, int n, float *loss,
                        float *grad);
/* iters Adam iterations at learning rate lr (one CUDA graph per iteration);
 * final_loss (may be NULL) receives the loss of the last iteration's forward */
int vefem_mlp_train(vefem_mlp *m, const float *X, const float *T, int n, int iters, float lr,
                    float *final_loss);
/* Adam moments and step count back to zero (parameters kept) */
int vefem_mlp_reset_optimizer(vefem_mlp *m);
int vefem_mlp_destroy(vefem_mlp *m);
const char *vefem_mlp_last_error(const vefem_mlp *m);

#ifdef __cplusplus
}
#endif

#endif /* VEFEM_H */
