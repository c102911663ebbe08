// Deterministic scatter of element contributions into the global residual and
// the AIJ values, in element order, without atomics.
//
// The reference adds element after element with VecSetValues/MatSetValues
// (ADD_VALUES, Storage_mod.F90:10-115), so a global entry is the sequential
// sum  ((v + c_e1) + c_e2) + ...  over the elements that touch it, in element
// order.  Here each global entry is owned by one thread, which reads the
// contributions from the element scratch through a precomputed contributor
// list sorted by element and adds them in that order: the same sum, bit for
// bit, with no colouring and no atomics.  These kernels are bandwidth-bound
// (the lists and the scratch are streamed once).
#include <cuda_runtime.h>
#include <stdint.h>

#include "vefem_internal.h"

namespace vefem {

// b[gnode*6 + jeq] += sum over contributors (e*9 + jnod) of rs[(e*9+jnod)*6 + jeq]
__global__ void k_gather_residual(const GatherArgs g, const double *__restrict__ rs,
                                  double *__restrict__ b)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nnodes * 6) return;
    const int node = (int)(t / 6), jeq = (int)(t - (int64_t)node * 6);
    const double acc0 = g.store ? 0.0 : b[t];
    b[t] = ordered_sum(acc0, g.ncon, g.nptr[node], g.nptr[node + 1],
                       [&](int c) { return rs[(int64_t)c * 6 + jeq]; });
}

// one thread per (node-pair block, jeq, ieq)
__global__ void k_gather_jacobian(const GatherArgs g, const double *__restrict__ es,
                                  double *__restrict__ vals)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nblocks * 36) return;
    const int blk = (int)(t / 36);
    const int r = (int)(t - (int64_t)blk * 36);
    const int jeq = r / 6, ieq = r - 6 * (r / 6);
    const int64_t slot = g.rowptr[(int64_t)g.brow[blk] * 6 + jeq] + g.boff[blk] + ieq;
    const double acc0 = g.store ? 0.0 : vals[slot];
    vals[slot] = ordered_sum(acc0, g.bcon, g.bptr[blk], g.bptr[blk + 1],
                             [&](int c) { return es[(int64_t)c * 36 + r]; });
}

// arclength column: the last entry of every node row (column N - 1)
__global__ void k_gather_arclength(const GatherArgs g, const double *__restrict__ as,
                                   double *__restrict__ vals)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nnodes * 6) return;
    const int node = (int)(t / 6), jeq = (int)(t - (int64_t)node * 6);
    const int64_t slot = g.rowptr[t + 1] - 1;
    const double acc0 = g.store ? 0.0 : vals[slot];
    vals[slot] = ordered_sum(acc0, g.ncon, g.nptr[node], g.nptr[node + 1],
                             [&](int c) { return as[(int64_t)c * 6 + jeq]; });
}

// Dirichlet rows: b = TL - value, and the AIJ row zeroed with 1 on the diagonal
template <class V>
__global__ void k_dirichlet(int nrows, int nnodes, const int64_t *__restrict__ rows,
                            const double *__restrict__ values, const double *__restrict__ TL,
                            double *b, const int64_t *__restrict__ rowptr,
                            const int32_t *__restrict__ colind, V *vals)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const int64_t row = rows[r];
    if (row < 0 || row >= (int64_t)nnodes * 6) return;   // rows outside the node unknowns are ignored
    if (b) {
        const int64_t node = row / 6, eq = row - 6 * (row / 6);
        b[row] = TL[eq * nnodes + node] - values[r];
    }
    if (vals) {
        for (int64_t s = rowptr[row]; s < rowptr[row + 1]; s++)
            vals[s] = colind[s] == row ? (V)1 : (V)0;
    }
}

cudaError_t launch_dirichlet(int nrows, int nnodes, const int64_t *rows, const double *values,
                             const double *TL, double *b, const int64_t *rowptr,
                             const int32_t *colind, void *vals, int vals_float, cudaStream_t s)
{
    if (nrows <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)((nrows + 127) / 128);
    if (vals_float)
        k_dirichlet<float><<<grid, 128, 0, s>>>(nrows, nnodes, rows, values, TL, b, rowptr, colind,
                                                 static_cast<float *>(vals));
    else
        k_dirichlet<double><<<grid, 128, 0, s>>>(nrows, nnodes, rows, values, TL, b, rowptr,
                                                  colind, static_cast<double *>(vals));
    return cudaGetLastError();
}

static inline unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

cudaError_t launch_gather_residual(const GatherArgs &g, const double *rs, double *b,
                                   cudaStream_t s)
{
    const int64_t n = (int64_t)g.nnodes * 6;
    if (n == 0) return cudaSuccess;
    k_gather_residual<<<grid_for(n, 256), 256, 0, s>>>(g, rs, b);
    return cudaGetLastError();
}

cudaError_t launch_gather_jacobian(const GatherArgs &g, const double *es, double *vals,
                                   cudaStream_t s)
{
    const int64_t n = (int64_t)g.nblocks * 36;
    if (n == 0) return cudaSuccess;
    k_gather_jacobian<<<grid_for(n, 288), 288, 0, s>>>(g, es, vals);
    return cudaGetLastError();
}

cudaError_t launch_gather_arclength(const GatherArgs &g, const double *as, double *vals,
                                    cudaStream_t s)
{
    const int64_t n = (int64_t)g.nnodes * 6;
    if (n == 0 || g.nex == 0) return cudaSuccess;
    k_gather_arclength<<<grid_for(n, 256), 256, 0, s>>>(g, as, vals);
    return cudaGetLastError();
}

}  // namespace vefem
