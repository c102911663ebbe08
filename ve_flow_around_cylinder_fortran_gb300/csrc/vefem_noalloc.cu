// Residual-only bulk assembly that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc when they assemble -- a
// host whose device memory is owned by another allocator (a PETSc/Kokkos
// memory pool, a framework that reserves the whole GPU at start-up), code
// that runs inside a section where allocation is forbidden (real-time
// loops), or hosts that cannot keep a library context alive between calls.
// vefem_assemble needs a context whose tables and scratch are allocated on
// the device; this entry point needs none: the caller passes device inputs
// and the device output, and the scratch (element residuals, node incidence
// lists) lives in one file-scope static device array of fixed size that
// every GPU loading the library holds until the process exits.
//
// Limits and rules:
//  * at most NOALLOC_MAX_EL elements and NOALLOC_MAX_NODES nodes per call
//    (about 17.7 MB of static scratch); larger meshes are rejected with
//    VEFEM_ERR_ARG before anything runs;
//  * at most NOALLOC_MAX_NODE_ELEMS elements may share one node, and every
//    connectivity id must lie in 1..nnodes; both are checked on the device
//    before anything is added into b, and a violation returns VEFEM_ERR_ARG
//    with b unchanged;
//  * the first call on a device, with that device current, looks up the
//    scratch array's device address (cudaGetSymbolAddress) and uploads the
//    Gauss tables; make that first call before any stream capture;
//  * every call waits for its stream to finish before it returns (it reads
//    the device-side error flag), and it leaves the caller's current device
//    as it found it;
//  * every call shares the one scratch array and leaves its contents behind;
//    the parts that must start at zero (the node counters, the error flag)
//    are cleared by the call itself.  Calls that overlap on the GPU (other
//    streams, other host threads) race on the scratch: serialise them.
//
// The result is the same, bit for bit, as vefem_assemble(VEFEM_RESIDUAL):
// element residuals from the same physics source, then per row an in-order
// (element-order) sum; the node incidence lists are built with atomic counters
// and each node's short list is sorted by element before summing.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "vefem.h"
#include "vefem_internal.h"
#include "vefem_physics.cuh"

namespace {

constexpr int NOALLOC_MAX_EL = 32768;
constexpr int NOALLOC_MAX_NODES = 9 * NOALLOC_MAX_EL;
constexpr int NOALLOC_MAX_DEVICES = 64;
constexpr int NOALLOC_MAX_NODE_ELEMS = 32;   // elements sharing one node

struct NoAllocScratch {
    double rs[NOALLOC_MAX_EL * 54];          // element residuals [(e*9 + jnod)*6 + jeq]
    int32_t cnt[NOALLOC_MAX_NODES + 1];      // per-node counters (cleared by every call)
    int32_t off[NOALLOC_MAX_NODES + 1];      // exclusive prefix sums of the counters
    int32_t list[NOALLOC_MAX_EL * 9];        // per-node (e*9 + jnod), unsorted
    int32_t err;                             // 1: a node has too many elements, 2: bad node id
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__constant__ double na_w[9];
__constant__ double na_bfn[9][9];
__constant__ double na_dfdc[9][9];
__constant__ double na_dfde[9][9];
__constant__ double na_d2fdc2[9][9];
__constant__ double na_d2fde2[9][9];
__constant__ double na_d2fdce[9][9];

constexpr int NA_EPB = 8;
constexpr int NA_THREADS = NA_EPB * 9;

struct NaView {
    const double *p;
    __device__ __forceinline__ double operator()(int pos) const { return p[pos]; }
};

// element residuals, thread = (element, Gauss point), in-order Gauss sum
template <int FORM>
__global__ void __launch_bounds__(NA_THREADS)
k_na_residual(int nel, int nnodes, const int32_t *conn, const double *xyz, const double *TL,
              const double *EU, const vefem::KParams prm, NoAllocScratch *S)
{
    __shared__ double s_tl[NA_EPB][54];
    __shared__ double s_part[NA_EPB][9][54];
    if (S->err) return;   // node ids failed validation in k_na_count
    const int t = threadIdx.x;
    const int el = t / 9;
    const int ig = t - el * 9;
    const int e = blockIdx.x * NA_EPB + el;
    const bool live = e < nel;
    for (int i = t; i < NA_EPB * 54; i += blockDim.x) {
        const int ee = blockIdx.x * NA_EPB + i / 54;
        const int pos = i - (i / 54) * 54;
        if (ee < nel) {
            const int inod = pos / 6, f = pos - 6 * (pos / 6);
            s_tl[i / 54][pos] = TL[(size_t)f * nnodes + (conn[(size_t)inod * nel + ee] - 1)];
        }
    }
    __syncthreads();
    if (live) {
        double x[9], y[9], dFx[9], dFy[9], d2x[9], d2y[9];
#pragma unroll
        for (int n = 0; n < 9; n++) {
            const int gn = conn[(size_t)n * nel + e] - 1;
            x[n] = xyz[gn];
            y[n] = xyz[nnodes + gn];
        }
        auto go = vefem::geometry(na_bfn[ig], na_dfdc[ig], na_dfde[ig], na_d2fdc2[ig],
                                  na_d2fde2[ig], na_d2fdce[ig], na_w[ig], x, y, dFx, dFy, d2x,
                                  d2y);
        double WiN = prm.WiN;
        if (prm.nex > 0) WiN = prm.Wi0 * EU[prm.nex - 1];
        NaView V{s_tl[el]};
        auto I = vefem::interpolate(V, na_bfn[ig], dFx, dFy, d2x, d2y);
        double dotU[9];
        auto g = vefem::gauss_point<FORM>(I, prm, WiN, go.H2, dFx, dFy, dotU);
#pragma unroll
        for (int n = 0; n < 9; n++)
            vefem::test_node<FORM>(g, prm, na_bfn[ig][n], dFx[n], dFy[n], dotU[n], go.WET,
                                   &s_part[el][ig][n * 6]);
    }
    __syncthreads();
    for (int i = t; i < NA_EPB * 54; i += blockDim.x) {
        const int le = i / 54, pos = i - (i / 54) * 54;
        const int ee = blockIdx.x * NA_EPB + le;
        if (ee >= nel) continue;
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 9; q++) s = s + s_part[le][q][pos];
        S->rs[(size_t)ee * 54 + pos] = s;
    }
}

__global__ void k_na_clear(int nnodes, NoAllocScratch *S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= nnodes) S->cnt[i] = 0;
    if (i == 0) S->err = 0;
}

// counts the elements of every node and validates the node ids
__global__ void k_na_count(int nel, int nnodes, const int32_t *conn, NoAllocScratch *S)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nel * 9) return;
    const int node = conn[t] - 1;
    if (node < 0 || node >= nnodes) {
        S->err = 2;
        return;
    }
    atomicAdd(&S->cnt[node], 1);
}

// single-CTA exclusive scan of cnt[0..nnodes) into off[0..nnodes], then clears cnt
__global__ void __launch_bounds__(1024) k_na_scan(int nnodes, NoAllocScratch *S)
{
    __shared__ int32_t s_sum[1024];
    const int t = threadIdx.x;
    const int per = (nnodes + 1023) / 1024;
    const int i0 = t * per;
    const int i1 = min(i0 + per, nnodes);
    int32_t local = 0;
    bool crowded = false;
    for (int i = i0; i < i1; i++) {
        local += S->cnt[i];
        crowded |= S->cnt[i] > NOALLOC_MAX_NODE_ELEMS;
    }
    // a node with too many elements fails the call before k_na_gather adds
    // anything into b (same value from every writer)
    if (crowded && S->err == 0) S->err = 1;
    s_sum[t] = local;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        const int32_t v = t >= d ? s_sum[t - d] : 0;
        __syncthreads();
        s_sum[t] += v;
        __syncthreads();
    }
    int32_t run = s_sum[t] - local;
    for (int i = i0; i < i1; i++) {
        S->off[i] = run;
        run += S->cnt[i];
    }
    if (t == 1023) S->off[nnodes] = s_sum[1023];
    __syncthreads();
    for (int i = i0; i < i1; i++) S->cnt[i] = 0;
}

__global__ void k_na_fill(int nel, const int32_t *conn, NoAllocScratch *S)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nel * 9 || S->err) return;
    const int jnod = t / nel, e = t - jnod * nel;   // conn is node-major [9][nel]
    const int node = conn[t] - 1;
    const int pos = atomicAdd(&S->cnt[node], 1);
    S->list[S->off[node] + pos] = e * 9 + jnod;
}

// b[node*6 + jeq] += element-ordered sum of the node's element residual rows
__global__ void k_na_gather(int nnodes, double *b, NoAllocScratch *S)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * 6 || S->err) return;   // b stays untouched on every error
    const int node = t / 6, jeq = t - 6 * (t / 6);
    const int c0 = S->off[node], n = S->off[node + 1] - c0;
    int32_t c[NOALLOC_MAX_NODE_ELEMS];
    for (int k = 0; k < n; k++) {
        const int32_t v = S->list[c0 + k];
        int j = k - 1;
        while (j >= 0 && c[j] > v) {
            c[j + 1] = c[j];
            j--;
        }
        c[j + 1] = v;
    }
    double acc = b[t];
    for (int k = 0; k < n; k++) acc = acc + S->rs[(size_t)c[k] * 6 + jeq];
    b[t] = acc;
}

std::mutex g_setup_mutex;
NoAllocScratch *g_scratch_ptr[NOALLOC_MAX_DEVICES] = {};

// once per device, with that device current: the scratch address and the tables
cudaError_t setup_device(int device, NoAllocScratch **out)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_ptr[device]) {
        *out = g_scratch_ptr[device];
        return cudaSuccess;
    }
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    vefem::GaussTables t;
    vefem::gauss_tables_host(&t);
    if ((e = cudaMemcpyToSymbol(na_w, t.w, sizeof(t.w))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(na_bfn, t.bfn, sizeof(t.bfn))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(na_dfdc, t.dfdc, sizeof(t.dfdc))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(na_dfde, t.dfde, sizeof(t.dfde))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(na_d2fdc2, t.d2fdc2, sizeof(t.d2fdc2))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(na_d2fde2, t.d2fde2, sizeof(t.d2fde2))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(na_d2fdce, t.d2fdce, sizeof(t.d2fdce))) != cudaSuccess) return e;
    g_scratch_ptr[device] = static_cast<NoAllocScratch *>(ptr);
    *out = g_scratch_ptr[device];
    return cudaSuccess;
}

int na_fail(int code, const std::string &msg)
{
    vefem::set_global_error(msg);
    return code;
}

}  // namespace

extern "C" int vefem_assemble_residual_noalloc(const vefem_params *params, int nnodes, int nel,
                                               const int32_t *conn, const double *xyz,
                                               const double *TL, const double *EU, double *b,
                                               void *stream)
{
    const char *me = "vefem_assemble_residual_noalloc: ";
    if (!params || !conn || !xyz || !TL || !b) return na_fail(VEFEM_ERR_ARG, std::string(me) + "NULL argument");
    if (params->nex < 0 || params->nex > 1 || (params->nex == 1 && !EU))
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "nex must be 0, or 1 with EU");
    if (params->form != VEFEM_FORM_T && params->form != VEFEM_FORM_SQRT)
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "form must be T or SQRT");
    if (params->model < 0 || params->model > 6)
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "model out of range");
    if (params->device < 0 || params->device >= NOALLOC_MAX_DEVICES)
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "device out of range");
    if (nel <= 0 || nnodes <= 0)
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "empty mesh");
    if (nel > NOALLOC_MAX_EL)
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "nel = " + std::to_string(nel) +
                                          " exceeds the static scratch limit of " +
                                          std::to_string(NOALLOC_MAX_EL) + " elements");
    if (nnodes > NOALLOC_MAX_NODES)
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "nnodes = " + std::to_string(nnodes) +
                                          " exceeds the static scratch limit of " +
                                          std::to_string(NOALLOC_MAX_NODES) + " nodes");
    int prev_device = -1;
    cudaError_t e = cudaGetDevice(&prev_device);
    if (e != cudaSuccess) return na_fail(VEFEM_ERR_CUDA, std::string(me) + cudaGetErrorString(e));
    // the caller's current device is restored on every return below
    struct DeviceGuard {
        int dev;
        ~DeviceGuard() { cudaSetDevice(dev); }
    } guard{prev_device};
    e = cudaSetDevice(params->device);
    NoAllocScratch *S = nullptr;
    if (e == cudaSuccess) e = setup_device(params->device, &S);
    if (e != cudaSuccess) return na_fail(VEFEM_ERR_CUDA, std::string(me) + cudaGetErrorString(e));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    vefem::KParams k;
    k.model = params->model; k.form = params->form; k.nex = params->nex;
    k.ReN = params->ReN; k.WiN = params->WiN; k.BvN = params->BvN; k.VeN = params->VeN;
    k.DfN = params->DfN; k.Wi0 = params->Wi0; k.dt = params->dt; k.eps = params->fd_eps;
    const int grid = (nel + NA_EPB - 1) / NA_EPB;
    k_na_clear<<<(nnodes + 1 + 255) / 256, 256, 0, s>>>(nnodes, S);
    k_na_count<<<(nel * 9 + 255) / 256, 256, 0, s>>>(nel, nnodes, conn, S);
    if (k.form == VEFEM_FORM_SQRT)
        k_na_residual<1><<<grid, NA_THREADS, 0, s>>>(nel, nnodes, conn, xyz, TL, EU, k, S);
    else
        k_na_residual<0><<<grid, NA_THREADS, 0, s>>>(nel, nnodes, conn, xyz, TL, EU, k, S);
    k_na_scan<<<1, 1024, 0, s>>>(nnodes, S);
    k_na_fill<<<(nel * 9 + 255) / 256, 256, 0, s>>>(nel, conn, S);
    k_na_gather<<<(nnodes * 6 + 255) / 256, 256, 0, s>>>(nnodes, b, S);
    int32_t err = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&err, &S->err, sizeof(err), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return na_fail(VEFEM_ERR_CUDA, std::string(me) + cudaGetErrorString(e));
    if (err == 2) return na_fail(VEFEM_ERR_ARG, std::string(me) + "connectivity id out of range");
    if (err)
        return na_fail(VEFEM_ERR_ARG, std::string(me) + "a node belongs to more than " +
                                          std::to_string(NOALLOC_MAX_NODE_ELEMS) + " elements");
    return VEFEM_OK;
}
