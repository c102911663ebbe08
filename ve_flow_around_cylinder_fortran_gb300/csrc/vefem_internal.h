// Internal interface between the C-ABI layer (vefem_capi.cu) and the kernel
// translation units.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace vefem {

enum { FORM_T = 0, FORM_SQRT = 1 };

// FP64 residual kernel: elements per CTA and per batched work item
constexpr int RES_EPB = 8;

// Specialisations that leave out terms which are exact zeros for the given
// parameters; a sum that drops an exact-zero addend keeps its value, so the
// results are the same as the general code (up to the sign of a zero result).
enum { SPEC_RE0 = 1,   // ReN == 0: convection, LSME-momentum and (ReN/dt, ReN*tsugn) terms
       SPEC_DF0 = 2 }; // DfN == 0: stress diffusion terms and DfN/Helem^2

// Physics parameters as the kernels read them (one copy per launch, by value).
struct KParams {
    int model, form, nex;
    double ReN, WiN, BvN, VeN, DfN, Wi0, dt, eps;
};

// Gauss-point tables of the 3x3 rule (Gauss_Quadrangle_mod.F90), [gp][node].
struct GaussTables {
    double w[9];
    double bfn[9][9], dfdc[9][9], dfde[9][9], d2fdc2[9][9], d2fde2[9][9], d2fdce[9][9];
    // outlet-edge tables: [edge 0..3][gp 0..2][node]
    double ew[3];
    double ebfn[4][3][9], edfdc[4][3][9], edfde[4][3][9], ed2c[4][3][9], ed2e[4][3][9],
        ed2ce[4][3][9];
};

void gauss_tables_host(GaussTables *t);

// Element-kernel arguments (device pointers).
struct ElemArgs {
    int nel, nnodes;
    const int32_t *conn;   // [9][nel], 0-based
    const double *xy;      // [2][nnodes]
    const double *TL;      // [6][nnodes]
    const double *EU;      // [nex] (device)
    double *rs;            // residual scratch [(e*9 + jnod)*6 + jeq]
    double *es;            // Jacobian scratch [((e*81 + jnod*9 + inod)*36 + jeq*6 + ieq]
    double *as;            // arclength-column scratch [(e*9 + jnod)*6 + jeq]
};

cudaError_t upload_tables(const GaussTables &t, cudaStream_t s);
cudaError_t launch_residual64(const ElemArgs &a, const KParams &p, cudaStream_t s);
cudaError_t launch_fd64(const ElemArgs &a, const KParams &p, cudaStream_t s);

// Outlet open-BC edges: residual and FD Jacobian of each listed edge into edge scratch.
struct EdgeArgs {
    int nedge, nel, nnodes;
    const int32_t *edge_elem;  // [nedge]
    const int32_t *edge_id;    // [nedge] 1..4
    const int32_t *conn;
    const double *xy, *TL, *EU;
    double *rs;                // [(k*9 + jnod)*6 + jeq]
    double *es;                // [((k*81 + jnod*9 + inod)*36 + jeq*6 + ieq]
    double *as;                // [(k*9 + jnod)*6 + jeq]
};
cudaError_t launch_edge64(const EdgeArgs &a, const KParams &p, int want_jac, cudaStream_t s);

// Deterministic element-ordered scatter (pull form).
struct GatherArgs {
    int nnodes;
    int nblocks;
    int nex;
    const int64_t *rowptr;     // [N+1]
    const int32_t *nptr;       // [nnodes+1] node -> residual contributors
    const int32_t *ncon;       // contributor = e*9 + jnod, element order
    const int32_t *brow;       // [nblocks] row node of each node-pair block
    const int32_t *boff;       // [nblocks] column offset of the block inside its rows
    const int32_t *bptr;       // [nblocks+1]
    const int32_t *bcon;       // contributor = e*81 + jnod*9 + inod, element order
    int store = 0;             // 1: the sums start from zero (VEFEM_ZERO_FIRST), the
                               // destination is written without being read
};
#ifdef __CUDACC__
// acc + val(con[c0]) + val(con[c0+1]) + ... in contributor order, the same
// sum as the plain loop, but the first ORDERED_PREFETCH contributor ids, then
// their values, are loaded before the first addition: independent loads in
// flight instead of an id -> value -> add chain per contributor.
constexpr int ORDERED_PREFETCH = 4;
template <class T, class F>
__device__ __forceinline__ T ordered_sum(T acc, const int32_t *__restrict__ con, int c0, int c1,
                                         F val)
{
    int id[ORDERED_PREFETCH];
    T v[ORDERED_PREFETCH];
#pragma unroll
    for (int k = 0; k < ORDERED_PREFETCH; k++) id[k] = c0 + k < c1 ? con[c0 + k] : 0;
#pragma unroll
    for (int k = 0; k < ORDERED_PREFETCH; k++) v[k] = c0 + k < c1 ? val(id[k]) : T(0);
#pragma unroll
    for (int k = 0; k < ORDERED_PREFETCH; k++)
        if (c0 + k < c1) acc = acc + v[k];
    for (int c = c0 + ORDERED_PREFETCH; c < c1; c++) acc = acc + val(con[c]);
    return acc;
}
#endif

cudaError_t launch_gather_residual(const GatherArgs &g, const double *rs, double *b,
                                   cudaStream_t s);
cudaError_t launch_gather_jacobian(const GatherArgs &g, const double *es, double *vals,
                                   cudaStream_t s);
cudaError_t launch_gather_arclength(const GatherArgs &g, const double *as, double *vals,
                                    cudaStream_t s);

// Exact-Jacobian kernels (vefem_exact.cu): element Jacobian and arclength column in T,
// launched through launch_exact_batched (declared below with the batched form).
cudaError_t upload_tables_exact(const GaussTables &t, cudaStream_t s);
cudaError_t launch_gather_jacobian32(const GatherArgs &g, const float *es, float *vals,
                                     cudaStream_t s);
cudaError_t launch_gather_arclength32(const GatherArgs &g, const float *as, float *vals,
                                      cudaStream_t s);

cudaError_t launch_dirichlet(int nrows, int nnodes, const int64_t *rows, const double *values,
                             const double *TL, double *b, const int64_t *rowptr,
                             const int32_t *colind, void *vals, int vals_float, cudaStream_t s);

// Message returned by vefem_last_error(NULL) for entry points without a context.
void set_global_error(const std::string &msg);

// ---- Batched form: many instances (mesh, pattern, parameters) in one launch.
// One descriptor per instance in device memory; the persistent kernels walk a
// list of work items (instance, first element, element count) with a grid
// stride.  FORM and the specialisation must be the same for all instances.
struct BatchInst {
    ElemArgs ea;          // element side (TL, EU, rs set per call)
    KParams prm;
    GatherArgs ga;
    void *es, *as;        // element Jacobian / arclength scratch (T of the launch)
    double *b;            // residual (device)
    void *vals;           // AIJ values (T of the launch)
};
struct WorkItem {
    int inst, e0, count, pad;
};
cudaError_t launch_residual64_batched(const BatchInst *insts, const WorkItem *work, int nwork,
                                      int form, int spec, int grid, cudaStream_t s);
template <class T>
cudaError_t launch_exact_batched(const BatchInst *insts, const WorkItem *work, int nwork,
                                 int form, int spec, int grid, cudaStream_t s);
// occupancy of the persistent kernels (resident CTAs per SM)
int exact_batched_ctas_per_sm(int elem_size, int form, int spec);
int residual_batched_ctas_per_sm(int form, int spec);

}  // namespace vefem
