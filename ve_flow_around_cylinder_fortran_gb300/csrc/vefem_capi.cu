// C-ABI layer of the element-assembly library (include/vefem.h).
//
// vefem_create turns one mesh and one frozen AIJ pattern into device tables:
//  * conn0 [9][nel] 0-based, xy [2][nnodes];
//  * per node: the (element, local node) pairs touching it, in element order
//    (residual rows and the arclength column);
//  * per node-pair block (row node gj, column node gi): the offset of column
//    gi*6 inside the six rows of gj (the six columns of a node are adjacent in
//    a sorted AIJ row) and the (element, jnod, inod) triples touching it, in
//    element order.
// With these, the scatter kernels sum every global entry in element order,
// which is what ADD_VALUES on one rank does (Storage_mod.F90:10-115).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "vefem.h"
#include "vefem_ctx.h"
#include "vefem_internal.h"

using namespace vefem;

static std::string g_create_error;

void vefem::set_global_error(const std::string &msg) { g_create_error = msg; }

namespace vefem {

// Gauss_Quadrangle_mod.F90: setQuadraticQuadrangle :405-478 (same expression
// order as the Fortran; host code is built with -ffp-contract=off)
static void q2_basis(double c, double e, double *bfn, double *dfdc, double *dfde, double *d2c,
                     double *d2e, double *d2ce)
{
    bfn[0] = +(1.0 - c) * c * (1.0 - e) * e / 4.0;
    bfn[1] = -(1.0 + c) * c * (1.0 - e) * e / 4.0;
    bfn[2] = +(1.0 + c) * c * (1.0 + e) * e / 4.0;
    bfn[3] = -(1.0 - c) * c * (1.0 + e) * e / 4.0;
    bfn[4] = -(1.0 + c) * (1.0 - c) * (1.0 - e) * e / 2.0;
    bfn[5] = +(1.0 + c) * c * (1.0 + e) * (1.0 - e) / 2.0;
    bfn[6] = +(1.0 + c) * (1.0 - c) * (1.0 + e) * e / 2.0;
    bfn[7] = -(1.0 - c) * c * (1.0 + e) * (1.0 - e) / 2.0;
    bfn[8] = +(1.0 + c) * (1.0 - c) * (1.0 + e) * (1.0 - e);
    dfdc[0] = +(1.0 - 2.0 * c) * (1.0 - e) * e / 4.0;
    dfdc[1] = -(1.0 + 2.0 * c) * (1.0 - e) * e / 4.0;
    dfdc[2] = +(1.0 + 2.0 * c) * (1.0 + e) * e / 4.0;
    dfdc[3] = -(1.0 - 2.0 * c) * (1.0 + e) * e / 4.0;
    dfdc[4] = -(-2.0 * c) * (1.0 - e) * e / 2.0;
    dfdc[5] = +(1.0 + 2.0 * c) * (1.0 + e) * (1.0 - e) / 2.0;
    dfdc[6] = +(-2.0 * c) * (1.0 + e) * e / 2.0;
    dfdc[7] = -(1.0 - 2.0 * c) * (1.0 + e) * (1.0 - e) / 2.0;
    dfdc[8] = +(-2.0 * c) * (1.0 + e) * (1.0 - e);
    d2c[0] = +(-2.0) * (1.0 - e) * e / 4.0;
    d2c[1] = -(+2.0) * (1.0 - e) * e / 4.0;
    d2c[2] = +(+2.0) * (1.0 + e) * e / 4.0;
    d2c[3] = -(-2.0) * (1.0 + e) * e / 4.0;
    d2c[4] = -(-2.0) * (1.0 - e) * e / 2.0;
    d2c[5] = +(+2.0) * (1.0 + e) * (1.0 - e) / 2.0;
    d2c[6] = +(-2.0) * (1.0 + e) * e / 2.0;
    d2c[7] = -(-2.0) * (1.0 + e) * (1.0 - e) / 2.0;
    d2c[8] = +(-2.0) * (1.0 + e) * (1.0 - e);
    d2ce[0] = +(1.0 - 2.0 * c) * (1.0 - 2.0 * e) / 4.0;
    d2ce[1] = -(1.0 + 2.0 * c) * (1.0 - 2.0 * e) / 4.0;
    d2ce[2] = +(1.0 + 2.0 * c) * (1.0 + 2.0 * e) / 4.0;
    d2ce[3] = -(1.0 - 2.0 * c) * (1.0 + 2.0 * e) / 4.0;
    d2ce[4] = -(-2.0 * c) * (1.0 - 2.0 * e) / 2.0;
    d2ce[5] = +(1.0 + 2.0 * c) * (-2.0 * e) / 2.0;
    d2ce[6] = +(-2.0 * c) * (1.0 + 2.0 * e) / 2.0;
    d2ce[7] = -(1.0 - 2.0 * c) * (-2.0 * e) / 2.0;
    d2ce[8] = +(-2.0 * c) * (-2.0 * e);
    dfde[0] = +(1.0 - c) * c * (1.0 - 2.0 * e) / 4.0;
    dfde[1] = -(1.0 + c) * c * (1.0 - 2.0 * e) / 4.0;
    dfde[2] = +(1.0 + c) * c * (1.0 + 2.0 * e) / 4.0;
    dfde[3] = -(1.0 - c) * c * (1.0 + 2.0 * e) / 4.0;
    dfde[4] = -(1.0 + c) * (1.0 - c) * (1.0 - 2.0 * e) / 2.0;
    dfde[5] = +(1.0 + c) * c * (-2.0 * e) / 2.0;
    dfde[6] = +(1.0 + c) * (1.0 - c) * (1.0 + 2.0 * e) / 2.0;
    dfde[7] = -(1.0 - c) * c * (-2.0 * e) / 2.0;
    dfde[8] = +(1.0 + c) * (1.0 - c) * (-2.0 * e);
    d2e[0] = +(1.0 - c) * c * (-2.0) / 4.0;
    d2e[1] = -(1.0 + c) * c * (-2.0) / 4.0;
    d2e[2] = +(1.0 + c) * c * (+2.0) / 4.0;
    d2e[3] = -(1.0 - c) * c * (+2.0) / 4.0;
    d2e[4] = -(1.0 + c) * (1.0 - c) * (-2.0) / 2.0;
    d2e[5] = +(1.0 + c) * c * (-2.0) / 2.0;
    d2e[6] = +(1.0 + c) * (1.0 - c) * (+2.0) / 2.0;
    d2e[7] = -(1.0 - c) * c * (-2.0) / 2.0;
    d2e[8] = +(1.0 + c) * (1.0 - c) * (-2.0);
}

// 3-point rule [0 + 1e-8, +sqrt(3/5), -sqrt(3/5)] (Gauss_Quadrangle_mod.F90:69-72),
// 2-D point order i (xi) outer, j (eta) inner (:82-101), weights :152-200.
void gauss_tables_host(GaussTables *t)
{
    double p1[3], w1[3];
    p1[0] = 0.0 + 1.0e-8;
    p1[1] = +std::sqrt(3.0 / 5.0);
    p1[2] = -std::sqrt(3.0 / 5.0);
    w1[0] = 8.0 / 9.0;
    w1[1] = 5.0 / 9.0;
    w1[2] = 5.0 / 9.0;
    int ng = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            t->w[ng] = w1[i] * w1[j];
            q2_basis(p1[i], p1[j], t->bfn[ng], t->dfdc[ng], t->dfde[ng], t->d2fdc2[ng],
                     t->d2fde2[ng], t->d2fdce[ng]);
            ng++;
        }
    // edge tables, setGaussBasisFunctionsQuadrangleEdge :243-314
    for (int ig = 0; ig < 3; ig++) t->ew[ig] = w1[ig];
    for (int ied = 0; ied < 4; ied++)
        for (int ig = 0; ig < 3; ig++) {
            double c, e;
            switch (ied) {
            case 0: c = p1[ig]; e = -1.0; break;
            case 1: c = +1.0; e = p1[ig]; break;
            case 2: c = p1[ig]; e = +1.0; break;
            default: c = -1.0; e = p1[ig]; break;
            }
            q2_basis(c, e, t->ebfn[ied][ig], t->edfdc[ied][ig], t->edfde[ied][ig],
                     t->ed2c[ied][ig], t->ed2e[ied][ig], t->ed2ce[ied][ig]);
        }
}

// edge contributions, sequential over edges (setEquationsEdge runs after the bulk)
template <class V>
__global__ void k_gather_edges(int nedge, int nex, const int64_t *rowptr, const int32_t *conn,
                               int nel, const int32_t *edge_elem, const int32_t *edge_row,
                               const int32_t *edge_off, const double *rs, const double *es,
                               const double *as, double *b, V *vals, int want_jac)
{
    for (int k = 0; k < nedge; k++) {
        const int e = edge_elem[k];
        for (int t = threadIdx.x; t < 54 + 2916 + 54; t += blockDim.x) {
            if (t < 54) {
                if (!b) continue;
                const int jnod = t / 6, jeq = t - 6 * (t / 6);
                const int64_t row = (int64_t)conn[jnod * nel + e] * 6 + jeq;
                b[row] = b[row] + rs[(int64_t)k * 54 + t];
            } else if (t < 54 + 2916) {
                if (!want_jac) continue;
                const int r = t - 54;
                const int blk = r / 36, q = r - 36 * (r / 36);
                const int jeq = q / 6, ieq = q - 6 * (q / 6);
                const int64_t slot = rowptr[(int64_t)edge_row[k * 81 + blk] * 6 + jeq] +
                                     edge_off[k * 81 + blk] + ieq;
                vals[slot] = vals[slot] + (V)es[(int64_t)k * 2916 + r];
            } else {
                if (!want_jac || nex == 0) continue;
                const int r = t - 54 - 2916;
                const int jnod = r / 6, jeq = r - 6 * (r / 6);
                const int64_t row = (int64_t)conn[jnod * nel + e] * 6 + jeq;
                const int64_t slot = rowptr[row + 1] - 1;
                vals[slot] = vals[slot] + (V)as[(int64_t)k * 54 + r];
            }
        }
        __syncthreads();
    }
}

}  // namespace vefem

// ---------------------------------------------------------------------------

static int fail(vefem_ctx *c, int code, const std::string &msg)
{
    if (c)
        c->err = msg;
    else
        g_create_error = msg;
    return code;
}

static int cuda_fail(vefem_ctx *c, cudaError_t e, const char *where)
{
    return fail(c, VEFEM_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                           \
    do {                                                                   \
        cudaError_t _e = (call);                                           \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, #call);           \
    } while (0)

template <class T>
static cudaError_t upload(T **dst, const T *src, size_t n, cudaStream_t s)
{
    cudaError_t e = cudaMalloc((void **)dst, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    if (n) e = cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s);
    return e;
}

static int check_params(const vefem_params *p, std::string &why)
{
    if (p->model < 0 || p->model > 6) { why = "model out of range"; return 0; }
    if (p->form != VEFEM_FORM_T && p->form != VEFEM_FORM_SQRT) { why = "form must be T or SQRT"; return 0; }
    if (p->nex < 0 || p->nex > 1) { why = "nex must be 0 or 1"; return 0; }
    if (!(p->fd_eps > 0.0)) { why = "fd_eps must be positive"; return 0; }
    if (p->device < 0) { why = "device must be >= 0"; return 0; }
    return 1;
}

static KParams to_kparams(const vefem_params *p)
{
    KParams k;
    k.model = p->model; k.form = p->form; k.nex = p->nex;
    k.ReN = p->ReN; k.WiN = p->WiN; k.BvN = p->BvN; k.VeN = p->VeN; k.DfN = p->DfN;
    k.Wi0 = p->Wi0; k.dt = p->dt; k.eps = p->fd_eps;
    return k;
}

// sorted-row search for column col in row r; -1 if absent
static int64_t find_col(const int64_t *rowptr, const int32_t *colind, int64_t r, int64_t col)
{
    const int32_t *b = colind + rowptr[r], *e = colind + rowptr[r + 1];
    const int32_t *it = std::lower_bound(b, e, (int32_t)col);
    if (it == e || *it != col) return -1;
    return (int64_t)(it - colind);
}

extern "C" int vefem_abi_version(void) { return VEFEM_ABI_VERSION; }

extern "C" int vefem_create(const vefem_mesh *mesh, const vefem_csr *pat,
                            const vefem_params *params, vefem_ctx **out)
{
    vefem_ctx *ctx = nullptr;
    if (!out) return fail(nullptr, VEFEM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!mesh || !pat || !params) return fail(nullptr, VEFEM_ERR_ARG, "NULL argument");
    if (mesh->nnodes <= 0 || mesh->nel <= 0 || !mesh->conn || !mesh->xyz)
        return fail(nullptr, VEFEM_ERR_ARG, "empty mesh");
    std::string why;
    if (!check_params(params, why)) return fail(nullptr, VEFEM_ERR_ARG, why);
    const int nn = mesh->nnodes, nel = mesh->nel, nex = params->nex;
    const int64_t N = (int64_t)nn * 6 + nex;
    if (pat->n != N || !pat->rowptr || !pat->colind)
        return fail(nullptr, VEFEM_ERR_ARG, "pattern size must be nnodes*6 + nex");
    if ((int64_t)nel * 81 >= (int64_t)INT32_MAX)
        return fail(nullptr, VEFEM_ERR_ARG, "too many elements for 32-bit contributor ids");
    const int64_t *rowptr = pat->rowptr;
    const int32_t *colind = pat->colind;
    if (rowptr[0] != 0) return fail(nullptr, VEFEM_ERR_PATTERN, "rowptr[0] must be 0");
    for (int64_t r = 0; r < N; r++)
        if (rowptr[r + 1] < rowptr[r]) return fail(nullptr, VEFEM_ERR_PATTERN, "rowptr decreasing");

    ctx = new (std::nothrow) vefem_ctx();
    if (!ctx) return fail(nullptr, VEFEM_ERR_NOMEM, "host allocation");
    ctx->device = params->device;
    ctx->nnodes = nn;
    ctx->nel = nel;
    ctx->nex = nex;
    ctx->N = N;
    ctx->nnz = rowptr[N];
    ctx->prm = to_kparams(params);

    // connectivity, 0-based, node-major [9][nel]
    std::vector<int32_t> conn0((size_t)9 * nel);
    for (int e = 0; e < nel; e++) {
        for (int i = 0; i < 9; i++) {
            int32_t g = mesh->conn[(size_t)i * nel + e];
            if (g < 1 || g > nn) {
                delete ctx;
                return fail(nullptr, VEFEM_ERR_ARG, "connectivity id out of range");
            }
            conn0[(size_t)i * nel + e] = g - 1;
        }
        for (int i = 0; i < 9; i++)
            for (int j = i + 1; j < 9; j++)
                if (conn0[(size_t)i * nel + e] == conn0[(size_t)j * nel + e]) {
                    delete ctx;
                    return fail(nullptr, VEFEM_ERR_ARG, "element with a repeated node");
                }
    }
    // node -> (element, local node), element order
    std::vector<int32_t> nptr(nn + 1, 0), ncon((size_t)nel * 9);
    for (int e = 0; e < nel; e++)
        for (int j = 0; j < 9; j++) nptr[conn0[(size_t)j * nel + e] + 1]++;
    for (int i = 0; i < nn; i++) nptr[i + 1] += nptr[i];
    {
        std::vector<int32_t> fill(nptr.begin(), nptr.end() - 1);
        for (int e = 0; e < nel; e++)
            for (int j = 0; j < 9; j++) ncon[fill[conn0[(size_t)j * nel + e]]++] = e * 9 + j;
    }
    // node-pair blocks: neighbours of each row node (from the elements), sorted
    std::vector<int32_t> nbptr(nn + 1, 0);
    std::vector<int32_t> nb;
    {
        std::vector<std::vector<int32_t>> adj(nn);
        for (int g = 0; g < nn; g++) adj[g].reserve(16);
        for (int e = 0; e < nel; e++)
            for (int j = 0; j < 9; j++) {
                const int gj = conn0[(size_t)j * nel + e];
                for (int i = 0; i < 9; i++) adj[gj].push_back(conn0[(size_t)i * nel + e]);
            }
        for (int g = 0; g < nn; g++) {
            auto &v = adj[g];
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
            nbptr[g + 1] = nbptr[g] + (int32_t)v.size();
        }
        nb.resize(nbptr[nn]);
        for (int g = 0; g < nn; g++) std::copy(adj[g].begin(), adj[g].end(), nb.begin() + nbptr[g]);
    }
    const int nblocks = nbptr[nn];
    std::vector<int32_t> brow(nblocks), boff(nblocks);
    for (int g = 0; g < nn; g++) {
        for (int q = nbptr[g]; q < nbptr[g + 1]; q++) {
            const int gi = nb[q];
            const int64_t r0 = (int64_t)g * 6;
            const int64_t s0 = find_col(rowptr, colind, r0, (int64_t)gi * 6);
            if (s0 < 0) {
                delete ctx;
                return fail(nullptr, VEFEM_ERR_PATTERN, "pattern lacks an element block");
            }
            const int64_t off = s0 - rowptr[r0];
            for (int jeq = 0; jeq < 6; jeq++) {
                const int64_t rs = rowptr[r0 + jeq];
                if (rs + off + 6 > rowptr[r0 + jeq + 1]) {
                    delete ctx;
                    return fail(nullptr, VEFEM_ERR_PATTERN, "pattern is not node-blocked");
                }
                for (int ieq = 0; ieq < 6; ieq++)
                    if (colind[rs + off + ieq] != gi * 6 + ieq) {
                        delete ctx;
                        return fail(nullptr, VEFEM_ERR_PATTERN, "pattern is not node-blocked");
                    }
            }
            brow[q] = g;
            boff[q] = (int32_t)off;
        }
    }
    // block contributors in element order
    std::vector<int32_t> bptr(nblocks + 1, 0), bcon((size_t)nel * 81);
    std::vector<int32_t> eblk((size_t)nel * 81);
    for (int e = 0; e < nel; e++)
        for (int j = 0; j < 9; j++) {
            const int gj = conn0[(size_t)j * nel + e];
            const int32_t *b0 = nb.data() + nbptr[gj], *b1 = nb.data() + nbptr[gj + 1];
            for (int i = 0; i < 9; i++) {
                const int gi = conn0[(size_t)i * nel + e];
                const int q = (int)(std::lower_bound(b0, b1, gi) - nb.data());
                eblk[(size_t)e * 81 + j * 9 + i] = q;
                bptr[q + 1]++;
            }
        }
    for (int q = 0; q < nblocks; q++) bptr[q + 1] += bptr[q];
    {
        std::vector<int32_t> fill(bptr.begin(), bptr.end() - 1);
        for (int e = 0; e < nel; e++)
            for (int r = 0; r < 81; r++) bcon[fill[eblk[(size_t)e * 81 + r]]++] = e * 81 + r;
    }
    if (nex) {
        for (int64_t r = 0; r < (int64_t)nn * 6; r++)
            if (rowptr[r + 1] == rowptr[r] || colind[rowptr[r + 1] - 1] != N - 1) {
                delete ctx;
                return fail(nullptr, VEFEM_ERR_PATTERN,
                            "with nex = 1 every node row must end with column N-1");
            }
    }
    // outlet edges
    const int nedge = mesh->n_outlet_edges > 0 ? mesh->n_outlet_edges : 0;
    std::vector<int32_t> erow((size_t)nedge * 81), eoff((size_t)nedge * 81);
    for (int k = 0; k < nedge; k++) {
        const int e = mesh->outlet_edge_elem[k];
        const int id = mesh->outlet_edge_id[k];
        if (e < 0 || e >= nel || id < 1 || id > 4) {
            delete ctx;
            return fail(nullptr, VEFEM_ERR_ARG, "outlet edge out of range");
        }
        for (int r = 0; r < 81; r++) {
            const int q = eblk[(size_t)e * 81 + r];
            erow[(size_t)k * 81 + r] = brow[q];
            eoff[(size_t)k * 81 + r] = boff[q];
        }
    }
    ctx->nblocks = nblocks;
    ctx->nedge = nedge;
    ctx->node_nnz = rowptr[(int64_t)nn * 6];
    ctx->blocks_cover = ctx->node_nnz == (int64_t)nblocks * 36 + (nex ? (int64_t)nn * 6 : 0);
    ctx->h_rowptr.assign(rowptr, rowptr + N + 1);
    ctx->h_colind.assign(colind, colind + rowptr[N]);

    cudaError_t ce = cudaSetDevice(ctx->device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&ctx->join, cudaEventDisableTiming);
    if (ce != cudaSuccess) {
        std::string m = std::string("cudaStreamCreate: ") + cudaGetErrorString(ce);
        delete ctx;
        return fail(nullptr, VEFEM_ERR_CUDA, m);
    }
    for (int i = 0; i < 8; i++) cudaEventCreate(&ctx->ev[i]);
    std::vector<double> xy((size_t)2 * nn);
    std::memcpy(xy.data(), mesh->xyz, sizeof(double) * nn);
    std::memcpy(xy.data() + nn, mesh->xyz + nn, sizeof(double) * nn);
    cudaStream_t s = ctx->stream;
    GaussTables tab;
    gauss_tables_host(&tab);
#define UPL(dst, src, n)                                                                      \
    if ((ce = upload(&ctx->dst, src, n, s)) != cudaSuccess) {                                 \
        std::string m = std::string("upload " #dst ": ") + cudaGetErrorString(ce);            \
        vefem_destroy(ctx);                                                                   \
        return fail(nullptr, VEFEM_ERR_CUDA, m);                                              \
    }
    UPL(d_conn, conn0.data(), conn0.size())
    UPL(d_xy, xy.data(), xy.size())
    UPL(d_rowptr, rowptr, (size_t)N + 1)
    UPL(d_colind, colind, (size_t)rowptr[N])
    UPL(d_nptr, nptr.data(), nptr.size())
    UPL(d_ncon, ncon.data(), ncon.size())
    UPL(d_brow, brow.data(), brow.size())
    UPL(d_boff, boff.data(), boff.size())
    UPL(d_bptr, bptr.data(), bptr.size())
    UPL(d_bcon, bcon.data(), bcon.size())
    if (nedge) {
        UPL(d_edge_elem, mesh->outlet_edge_elem, (size_t)nedge)
        UPL(d_edge_id, mesh->outlet_edge_id, (size_t)nedge)
        UPL(d_edge_row, erow.data(), erow.size())
        UPL(d_edge_off, eoff.data(), eoff.size())
    }
#undef UPL
    if ((ce = upload_tables(tab, s)) != cudaSuccess || (ce = upload_tables_exact(tab, s)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(s)) != cudaSuccess) {
        std::string m = std::string("tables: ") + cudaGetErrorString(ce);
        vefem_destroy(ctx);
        return fail(nullptr, VEFEM_ERR_CUDA, m);
    }
    *out = ctx;
    return VEFEM_OK;
}

extern "C" int vefem_set_params(vefem_ctx *ctx, const vefem_params *p)
{
    if (!ctx || !p) return VEFEM_ERR_ARG;
    std::string why;
    if (!check_params(p, why)) return fail(ctx, VEFEM_ERR_ARG, why);
    if (p->nex != ctx->nex) return fail(ctx, VEFEM_ERR_ARG, "nex is fixed by the pattern");
    if (p->device != ctx->device) return fail(ctx, VEFEM_ERR_ARG, "device is fixed at create");
    ctx->prm = to_kparams(p);
    return VEFEM_OK;
}

static cudaError_t ensure(double **p, size_t n)
{
    if (*p) return cudaSuccess;
    return cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(double));
}

extern "C" int vefem_assemble(vefem_ctx *ctx, const double *TL, const double *EU, int flags,
                              double *b, void *vals_v, int on_device)
{
    if (!ctx) return VEFEM_ERR_ARG;
    const int known = VEFEM_RESIDUAL | VEFEM_JAC_FD64 | VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32 |
                      VEFEM_ZERO_FIRST | VEFEM_OUTLET_EDGES | VEFEM_TIMING;
    if (flags & ~known) return fail(ctx, VEFEM_ERR_UNSUPPORTED, "unknown flag");
    const int jmode = flags & (VEFEM_JAC_FD64 | VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32);
    if (jmode && (jmode & (jmode - 1)))
        return fail(ctx, VEFEM_ERR_ARG, "at most one Jacobian flag");
    const bool want_res = flags & VEFEM_RESIDUAL;
    const bool want_jac = jmode != 0;
    const bool jac32 = jmode == VEFEM_JAC_EXACT32;
    const size_t vsize = jac32 ? sizeof(float) : sizeof(double);
    double *vals = jac32 ? nullptr : static_cast<double *>(vals_v);
    float *vals32 = jac32 ? static_cast<float *>(vals_v) : nullptr;
    const bool edges = (flags & VEFEM_OUTLET_EDGES) && ctx->nedge > 0;
    const bool timing = flags & VEFEM_TIMING;
    if (!want_res && !want_jac) return fail(ctx, VEFEM_ERR_ARG, "nothing requested");
    if (!TL) return fail(ctx, VEFEM_ERR_ARG, "TL is NULL");
    if (ctx->nex > 0 && !EU) return fail(ctx, VEFEM_ERR_ARG, "EU is NULL with nex = 1");
    if (want_res && !b) return fail(ctx, VEFEM_ERR_ARG, "b is NULL");
    if (want_jac && !vals_v) return fail(ctx, VEFEM_ERR_ARG, "vals is NULL");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t nel = ctx->nel, nn = ctx->nnodes;
    ctx->launches = 0;
    for (int i = 0; i < 5; i++) ctx->timing[i] = 0.0f;

    CK(ensure(&ctx->d_rs, nel * 54));
    if (want_jac && !jac32) {
        CK(ensure(&ctx->d_es, nel * 2916));
        if (ctx->nex) CK(ensure(&ctx->d_as, nel * 54));
    }
    if (jac32) {
        if (!ctx->d_es32) CK(cudaMalloc((void **)&ctx->d_es32, nel * 2916 * sizeof(float)));
        if (ctx->nex && !ctx->d_as32) CK(cudaMalloc((void **)&ctx->d_as32, nel * 54 * sizeof(float)));
    }
    if (edges) {
        CK(ensure(&ctx->d_ers, (size_t)ctx->nedge * 54));
        CK(ensure(&ctx->d_ees, (size_t)ctx->nedge * 2916));
        CK(ensure(&ctx->d_eas, (size_t)ctx->nedge * 54));
    }
    const double *dTL = TL, *dEU = EU;
    double *db = b, *dvals = vals;
    float *dvals32 = vals32;
    if (timing) CK(cudaEventRecord(ctx->ev[0], s));
    if (!on_device) {
        CK(ensure(&ctx->d_TL, nn * 6));
        CK(cudaMemcpyAsync(ctx->d_TL, TL, nn * 6 * sizeof(double), cudaMemcpyHostToDevice, s));
        dTL = ctx->d_TL;
        if (ctx->nex) {
            CK(ensure(&ctx->d_EU, 1));
            CK(cudaMemcpyAsync(ctx->d_EU, EU, sizeof(double), cudaMemcpyHostToDevice, s));
            dEU = ctx->d_EU;
        }
        if (want_res) {
            CK(ensure(&ctx->d_b, (size_t)ctx->N));
            db = ctx->d_b;
            if (!(flags & VEFEM_ZERO_FIRST))
                CK(cudaMemcpyAsync(db, b, ctx->N * sizeof(double), cudaMemcpyHostToDevice, s));
        }
        if (want_jac && !jac32) {
            CK(ensure(&ctx->d_vals, (size_t)ctx->nnz));
            dvals = ctx->d_vals;
            if (!(flags & VEFEM_ZERO_FIRST))
                CK(cudaMemcpyAsync(dvals, vals, ctx->nnz * sizeof(double), cudaMemcpyHostToDevice, s));
        }
        if (jac32) {
            if (!ctx->d_vals32) CK(cudaMalloc((void **)&ctx->d_vals32, ctx->nnz * sizeof(float)));
            dvals32 = ctx->d_vals32;
            if (!(flags & VEFEM_ZERO_FIRST))
                CK(cudaMemcpyAsync(dvals32, vals32, ctx->nnz * sizeof(float), cudaMemcpyHostToDevice, s));
        }
    }
    // VEFEM_ZERO_FIRST: the scatter writes the node rows' sums without reading
    // them (they start from zero, the same bits as after a memset); only what
    // it does not cover is cleared: the arclength rows, and every entry when
    // the caller's pattern has node-row entries outside the element blocks
    const bool zero_first = (flags & VEFEM_ZERO_FIRST) != 0;
    const int64_t nrow_nodes = (int64_t)ctx->nnodes * 6;
    if (zero_first) {
        if (want_res && ctx->N > nrow_nodes)
            CK(cudaMemsetAsync(db + nrow_nodes, 0, (ctx->N - nrow_nodes) * sizeof(double), s));
        if (want_jac) {
            const int64_t z0 = ctx->blocks_cover ? ctx->node_nnz : 0;
            char *base = jac32 ? (char *)dvals32 : (char *)dvals;
            if (ctx->nnz > z0) CK(cudaMemsetAsync(base + z0 * vsize, 0, (ctx->nnz - z0) * vsize, s));
        }
    }
    if (timing) CK(cudaEventRecord(ctx->ev[1], s));

    ElemArgs ea;
    ea.nel = ctx->nel;
    ea.nnodes = ctx->nnodes;
    ea.conn = ctx->d_conn;
    ea.xy = ctx->d_xy;
    ea.TL = dTL;
    ea.EU = dEU;
    ea.rs = ctx->d_rs;
    ea.es = ctx->d_es;
    ea.as = ctx->d_as;
    if (jmode == VEFEM_JAC_FD64) {
        CK(launch_fd64(ea, ctx->prm, s));
        ctx->launches++;
    } else {
        // The FP64 residual and an exact Jacobian are independent until the
        // scatter: the residual runs on a second stream, so the FP64 pipe works
        // on it while the exact kernel keeps the FP32 pipes busy.
        const bool side = want_res && want_jac;
        if (want_res) {
            if (side) {
                CK(cudaEventRecord(ctx->fork, s));
                CK(cudaStreamWaitEvent(ctx->stream2, ctx->fork, 0));
                CK(launch_residual64(ea, ctx->prm, ctx->stream2));
                CK(cudaEventRecord(ctx->join, ctx->stream2));
            } else {
                CK(launch_residual64(ea, ctx->prm, s));
            }
            ctx->launches++;
        }
        if (jmode == VEFEM_JAC_EXACT64 || jac32) {
            if (!ctx->d_self) {
                CK(cudaMalloc((void **)&ctx->d_self, sizeof(BatchInst)));
                std::vector<WorkItem> w(nel);
                for (int e = 0; e < (int)nel; e++) w[e] = {0, e, 1, 0};
                CK(cudaMalloc((void **)&ctx->d_work, nel * sizeof(WorkItem)));
                CK(cudaMemcpy(ctx->d_work, w.data(), nel * sizeof(WorkItem), cudaMemcpyHostToDevice));
                CK(cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device));
            }
            BatchInst &I = ctx->h_self;
            I.ea = ea;
            I.prm = ctx->prm;
            I.es = jac32 ? (void *)ctx->d_es32 : (void *)ctx->d_es;
            I.as = jac32 ? (void *)ctx->d_as32 : (void *)ctx->d_as;
            CK(cudaMemcpyAsync(ctx->d_self, &I, sizeof(BatchInst), cudaMemcpyHostToDevice, s));
            const int spec = (ctx->prm.ReN == 0.0 ? SPEC_RE0 : 0) | (ctx->prm.DfN == 0.0 ? SPEC_DF0 : 0);
            const int occ = exact_batched_ctas_per_sm(jac32 ? 4 : 8, ctx->prm.form, spec);
            const int grid = std::min<int>((int)nel, ctx->sms * std::max(1, occ));
            if (jac32)
                CK(launch_exact_batched<float>(ctx->d_self, ctx->d_work, (int)nel, ctx->prm.form, spec, grid, s));
            else
                CK(launch_exact_batched<double>(ctx->d_self, ctx->d_work, (int)nel, ctx->prm.form, spec, grid, s));
            ctx->launches++;
        }
        if (side) CK(cudaStreamWaitEvent(s, ctx->join, 0));
    }
    if (timing) CK(cudaEventRecord(ctx->ev[2], s));

    GatherArgs ga;
    ga.nnodes = ctx->nnodes;
    ga.nblocks = ctx->nblocks;
    ga.nex = ctx->nex;
    ga.rowptr = ctx->d_rowptr;
    ga.nptr = ctx->d_nptr;
    ga.ncon = ctx->d_ncon;
    ga.brow = ctx->d_brow;
    ga.boff = ctx->d_boff;
    ga.bptr = ctx->d_bptr;
    ga.bcon = ctx->d_bcon;
    ga.store = zero_first ? 1 : 0;
    if (want_res) {
        CK(launch_gather_residual(ga, ctx->d_rs, db, s));
        ctx->launches++;
    }
    if (timing) CK(cudaEventRecord(ctx->ev[3], s));
    ga.store = zero_first && ctx->blocks_cover ? 1 : 0;
    if (want_jac && !jac32) {
        CK(launch_gather_jacobian(ga, ctx->d_es, dvals, s));
        ctx->launches++;
        if (ctx->nex) {
            CK(launch_gather_arclength(ga, ctx->d_as, dvals, s));
            ctx->launches++;
        }
    }
    if (jac32) {
        CK(launch_gather_jacobian32(ga, ctx->d_es32, dvals32, s));
        ctx->launches++;
        if (ctx->nex) {
            CK(launch_gather_arclength32(ga, ctx->d_as32, dvals32, s));
            ctx->launches++;
        }
    }
    if (timing) CK(cudaEventRecord(ctx->ev[4], s));
    if (edges) {
        EdgeArgs eg;
        eg.nedge = ctx->nedge;
        eg.nel = ctx->nel;
        eg.nnodes = ctx->nnodes;
        eg.edge_elem = ctx->d_edge_elem;
        eg.edge_id = ctx->d_edge_id;
        eg.conn = ctx->d_conn;
        eg.xy = ctx->d_xy;
        eg.TL = dTL;
        eg.EU = dEU;
        eg.rs = ctx->d_ers;
        eg.es = ctx->d_ees;
        eg.as = ctx->d_eas;
        CK(launch_edge64(eg, ctx->prm, want_jac ? 1 : 0, s));
        if (jac32)
            k_gather_edges<float><<<1, 1024, 0, s>>>(
                ctx->nedge, ctx->nex, ctx->d_rowptr, ctx->d_conn, ctx->nel, ctx->d_edge_elem,
                ctx->d_edge_row, ctx->d_edge_off, ctx->d_ers, ctx->d_ees, ctx->d_eas,
                want_res ? db : nullptr, dvals32, 1);
        else
            k_gather_edges<double><<<1, 1024, 0, s>>>(
                ctx->nedge, ctx->nex, ctx->d_rowptr, ctx->d_conn, ctx->nel, ctx->d_edge_elem,
                ctx->d_edge_row, ctx->d_edge_off, ctx->d_ers, ctx->d_ees, ctx->d_eas,
                want_res ? db : nullptr, want_jac ? dvals : nullptr, want_jac ? 1 : 0);
        CK(cudaGetLastError());
        ctx->launches += 2;
    }
    if (timing) CK(cudaEventRecord(ctx->ev[5], s));
    if (!on_device) {
        if (want_res)
            CK(cudaMemcpyAsync(b, db, ctx->N * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (want_jac && !jac32)
            CK(cudaMemcpyAsync(vals, dvals, ctx->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (jac32)
            CK(cudaMemcpyAsync(vals32, dvals32, ctx->nnz * sizeof(float), cudaMemcpyDeviceToHost, s));
    }
    if (timing) CK(cudaEventRecord(ctx->ev[6], s));
    CK(cudaStreamSynchronize(s));
    if (timing) {
        float t01, t12, t23, t34, t45, t56;
        cudaEventElapsedTime(&t01, ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&t23, ctx->ev[2], ctx->ev[3]);
        cudaEventElapsedTime(&t34, ctx->ev[3], ctx->ev[4]);
        cudaEventElapsedTime(&t45, ctx->ev[4], ctx->ev[5]);
        cudaEventElapsedTime(&t56, ctx->ev[5], ctx->ev[6]);
        ctx->timing[0] = t12;
        ctx->timing[1] = t23;
        ctx->timing[2] = t34;
        ctx->timing[3] = t45;
        ctx->timing[4] = t01 + t56;
    }
    return VEFEM_OK;
}

extern "C" int vefem_apply_dirichlet(vefem_ctx *ctx, int nrows, const int64_t *rows,
                                     const double *values, const double *TL, double *b,
                                     void *vals, int flags, int on_device)
{
    if (!ctx) return VEFEM_ERR_ARG;
    const int jmode = flags & (VEFEM_JAC_FD64 | VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32);
    if (jmode && (jmode & (jmode - 1))) return fail(ctx, VEFEM_ERR_ARG, "at most one Jacobian flag");
    const bool want_res = flags & VEFEM_RESIDUAL;
    if (nrows < 0 || (nrows > 0 && (!rows || !values))) return fail(ctx, VEFEM_ERR_ARG, "bad rows");
    if (want_res && (!b || !TL)) return fail(ctx, VEFEM_ERR_ARG, "b or TL is NULL");
    if (jmode && !vals) return fail(ctx, VEFEM_ERR_ARG, "vals is NULL");
    const bool f32 = jmode == VEFEM_JAC_EXACT32;
    const int64_t nd = (int64_t)ctx->nnodes * 6;
    if (!on_device) {
        for (int r = 0; r < nrows; r++)
            if (rows[r] < 0 || rows[r] >= nd) return fail(ctx, VEFEM_ERR_ARG, "Dirichlet row out of range");
        for (int r = 0; r < nrows; r++) {
            const int64_t row = rows[r];
            if (want_res) b[row] = TL[(row % 6) * ctx->nnodes + row / 6] - values[r];
            if (jmode)
                for (int64_t s = ctx->h_rowptr[row]; s < ctx->h_rowptr[row + 1]; s++) {
                    const bool diag = ctx->h_colind[s] == row;
                    if (f32)
                        static_cast<float *>(vals)[s] = diag ? 1.0f : 0.0f;
                    else
                        static_cast<double *>(vals)[s] = diag ? 1.0 : 0.0;
                }
        }
        return VEFEM_OK;
    }
    CK(cudaSetDevice(ctx->device));
    CK(launch_dirichlet(nrows, ctx->nnodes, rows, values, TL, want_res ? b : nullptr,
                        ctx->d_rowptr, ctx->d_colind, jmode ? vals : nullptr, f32 ? 1 : 0,
                        ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return VEFEM_OK;
}

extern "C" int vefem_last_timing(const vefem_ctx *ctx, float *t, int n)
{
    if (!ctx || !t) return VEFEM_ERR_ARG;
    for (int i = 0; i < n && i < 5; i++) t[i] = ctx->timing[i];
    return VEFEM_OK;
}

extern "C" int vefem_last_launch_count(const vefem_ctx *ctx) { return ctx ? ctx->launches : -1; }

extern "C" void *vefem_stream(const vefem_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int vefem_destroy(vefem_ctx *ctx)
{
    if (!ctx) return VEFEM_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    void *ptrs[] = {ctx->d_conn, ctx->d_xy, ctx->d_rowptr, ctx->d_nptr, ctx->d_ncon, ctx->d_brow,
                    ctx->d_boff, ctx->d_bptr, ctx->d_bcon, ctx->d_edge_elem, ctx->d_edge_id,
                    ctx->d_edge_row, ctx->d_edge_off, ctx->d_rs, ctx->d_es, ctx->d_as,
                    ctx->d_ers, ctx->d_ees, ctx->d_eas, ctx->d_TL, ctx->d_EU, ctx->d_b,
                    ctx->d_vals, ctx->d_es32, ctx->d_as32, ctx->d_vals32, ctx->d_colind,
                    ctx->d_self, ctx->d_work, ctx->d_rowptr10, ctx->d_boff10, ctx->d_ses,
                    ctx->d_tlb, ctx->d_kw, ctx->d_Aptr, ctx->d_Astage, ctx->d_Bstage};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int i = 0; i < 8; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->join) cudaEventDestroy(ctx->join);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return VEFEM_OK;
}

extern "C" const char *vefem_last_error(const vefem_ctx *ctx)
{
    return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

// preAllocatePetsc (Petsc_mod.F90:629-743) restated for hosts without PETSc
extern "C" int vefem_build_pattern(const vefem_mesh *mesh, int nex, int64_t *n, int64_t *nnz,
                                   int64_t *rowptr, int32_t *colind)
{
    if (!mesh || !n || !nnz || mesh->nnodes <= 0 || mesh->nel <= 0 || nex < 0 || nex > 1)
        return fail(nullptr, VEFEM_ERR_ARG, "bad arguments to vefem_build_pattern");
    const int nn = mesh->nnodes, nel = mesh->nel;
    std::vector<std::vector<int32_t>> adj(nn);
    for (int e = 0; e < nel; e++)
        for (int j = 0; j < 9; j++) {
            const int gj = mesh->conn[(size_t)j * nel + e] - 1;
            if (gj < 0 || gj >= nn) return fail(nullptr, VEFEM_ERR_ARG, "connectivity id out of range");
            for (int i = 0; i < 9; i++) adj[gj].push_back(mesh->conn[(size_t)i * nel + e] - 1);
        }
    int64_t total = 0;
    for (int g = 0; g < nn; g++) {
        auto &v = adj[g];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        total += 6 * ((int64_t)v.size() * 6 + nex);
    }
    const int64_t N = (int64_t)nn * 6 + nex;
    if (nex) total += N;
    *n = N;
    *nnz = total;
    if (!rowptr || !colind) return VEFEM_OK;
    int64_t p = 0;
    rowptr[0] = 0;
    for (int g = 0; g < nn; g++)
        for (int jeq = 0; jeq < 6; jeq++) {
            for (int32_t gi : adj[g])
                for (int ieq = 0; ieq < 6; ieq++) colind[p++] = gi * 6 + ieq;
            if (nex) colind[p++] = (int32_t)(N - 1);
            rowptr[(int64_t)g * 6 + jeq + 1] = p;
        }
    if (nex) {
        for (int64_t c = 0; c < N; c++) colind[p++] = (int32_t)c;
        rowptr[N] = p;
    }
    return VEFEM_OK;
}
