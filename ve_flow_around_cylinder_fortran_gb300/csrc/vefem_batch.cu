// Batched form of the bulk assembly: many instances in one persistent launch
// per kernel, captured once in a CUDA graph and replayed.
//
// Each instance keeps the tables of a single-mesh context (vefem_create); the
// batch adds one descriptor per instance in device memory (BatchInst) and a
// work list of (instance, first element, count) items for the element
// kernels, which run with a grid of SMs x resident CTAs and walk the work list
// with a grid stride; the element-batch tile (elements per work item) is
// chosen per mesh-size class by the autotuner.  The scatter is one persistent
// launch too: a work list of (instance, kind, first entry, count) items built
// at create, each item a run of entries of one instance's residual, Jacobian
// blocks or arclength column, so a CTA reads its instance's tables once per
// item and no thread searches for its instance.  Every global entry is still
// the element-ordered sum of the single-mesh gather, bit for bit; with
// VEFEM_ZERO_FIRST the sums start from zero in place of a memset of b and the
// AIJ values (the extra items clear the rows the gathers do not own: the
// lambda row and the lambda entry of b).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "vefem.h"
#include "vefem_ctx.h"
#include "vefem_internal.h"

using namespace vefem;

namespace {

const int EX_TILES[] = {1, 2, 4, 8};         // candidate element-batch tiles of the Jacobian kernel

// scatter work items: a run of entries of one kind of one instance
enum { SC_RES = 0, SC_JAC = 1, SC_ARC = 2, SC_EXTRA = 3 };
struct ScatterItem {
    int inst, kind;
    int64_t first;
    int count, pad;
};
constexpr int SC_RES_RUN = 2048;     // residual / arclength entries per item
constexpr int SC_JAC_RUN = 64 * 36;  // Jacobian entries (64 node-pair blocks) per item
constexpr int SC_THREADS = 256;

// One launch for the scatter of every instance: per item the instance's
// tables, then the element-ordered sums of the single-mesh gathers
// (vefem_gather.cu, vefem_exact.cu).  store: start each sum from zero
// (VEFEM_ZERO_FIRST) instead of the array's value.
template <class T>
__global__ void __launch_bounds__(SC_THREADS)
k_scatter_batched(const BatchInst *__restrict__ insts, const ScatterItem *__restrict__ items,
                  int nitems, int want_res, int want_jac, int store)
{
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const ScatterItem it = items[w];
        if ((it.kind == SC_RES && !want_res) || ((it.kind == SC_JAC || it.kind == SC_ARC) && !want_jac) ||
            (it.kind == SC_EXTRA && !store))
            continue;
        const BatchInst &I = insts[it.inst];
        const GatherArgs g = I.ga;
        const int64_t end = it.first + it.count;
        if (it.kind == SC_RES) {
            const double *rs = I.ea.rs;
            double *b = I.b;
            for (int64_t t = it.first + threadIdx.x; t < end; t += SC_THREADS) {
                const int node = (int)(t / 6), jeq = (int)(t - (int64_t)node * 6);
                double acc = store ? 0.0 : b[t];
                const int c0 = g.nptr[node], c1 = g.nptr[node + 1];
                for (int c = c0; c < c1; c++) acc = acc + rs[(int64_t)g.ncon[c] * 6 + jeq];
                b[t] = acc;
            }
        } else if (it.kind == SC_JAC) {
            const T *es = static_cast<const T *>(I.es);
            T *vals = static_cast<T *>(I.vals);
            for (int64_t t = it.first + threadIdx.x; t < end; t += SC_THREADS) {
                const int blk = (int)(t / 36);
                const int r = (int)(t - (int64_t)blk * 36);
                const int jeq = r / 6, ieq = r - 6 * (r / 6);
                const int64_t slot = g.rowptr[(int64_t)g.brow[blk] * 6 + jeq] + g.boff[blk] + ieq;
                T acc = store ? (T)0 : vals[slot];
                const int c0 = g.bptr[blk], c1 = g.bptr[blk + 1];
                for (int c = c0; c < c1; c++) acc = acc + es[(int64_t)g.bcon[c] * 36 + r];
                vals[slot] = acc;
            }
        } else if (it.kind == SC_ARC) {
            const T *as = static_cast<const T *>(I.as);
            T *vals = static_cast<T *>(I.vals);
            for (int64_t t = it.first + threadIdx.x; t < end; t += SC_THREADS) {
                const int node = (int)(t / 6), jeq = (int)(t - (int64_t)node * 6);
                const int64_t slot = g.rowptr[t + 1] - 1;
                T acc = store ? (T)0 : vals[slot];
                const int c0 = g.nptr[node], c1 = g.nptr[node + 1];
                for (int c = c0; c < c1; c++) acc = acc + as[(int64_t)g.ncon[c] * 6 + jeq];
                vals[slot] = acc;
            }
        } else {
            // the rows after the node unknowns: the lambda row of the values
            // (entries first .. end) and the lambda entries of b
            const int64_t n6 = (int64_t)g.nnodes * 6;
            if (want_jac) {
                T *vals = static_cast<T *>(I.vals);
                for (int64_t t = it.first + threadIdx.x; t < end; t += SC_THREADS) vals[t] = (T)0;
            }
            if (want_res && threadIdx.x < g.nex) I.b[n6 + threadIdx.x] = 0.0;
        }
    }
}

int size_class(int nel)
{
    int c = 0;
    for (int64_t lim = 2000; c < VEFEM_BATCH_CLASSES - 1 && nel >= lim; lim *= 2) c++;
    return c;
}

struct GraphKey {
    int flags = -1;
    std::vector<const void *> ptrs;
    bool operator==(const GraphKey &o) const { return flags == o.flags && ptrs == o.ptrs; }
};

}  // namespace

struct vefem_batch {
    int device = 0, ninst = 0, form = 0, spec = 0, nex = 0;
    int sms = 0;
    std::vector<vefem_ctx *> ctx;
    cudaStream_t s = nullptr, s2 = nullptr;   // s2: the FP64 residual beside the exact Jacobian
    cudaEvent_t ev[4] = {};
    cudaEvent_t fork = nullptr, join = nullptr;
    float timing[3] = {0, 0, 0};
    int launches = 0;
    int64_t replays = 0;
    std::string err;
    // per-class tiles
    int tiles[VEFEM_BATCH_CLASSES] = {1, 1, 1, 1, 1, 1};
    // descriptors and index spaces
    std::vector<BatchInst> h_inst;
    BatchInst *d_inst = nullptr;
    WorkItem *d_res_work = nullptr, *d_ex_work = nullptr;
    int n_res_work = 0, n_ex_work = 0;
    ScatterItem *d_sc_work = nullptr;
    int n_sc_work = 0;
    int64_t total_el = 0;
    // scratch
    double *d_rs = nullptr;
    void *d_es = nullptr, *d_as = nullptr;
    size_t es_elem = 0;                       // element size the Jacobian scratch holds
    // host-buffer staging
    std::vector<double *> st_TL, st_EU, st_b;
    std::vector<void *> st_vals;
    size_t st_vals_elem = 0;
    // graph
    cudaGraphExec_t graph = nullptr;
    GraphKey key;
};

namespace {

int bfail(vefem_batch *b, int code, const std::string &msg)
{
    if (b)
        b->err = msg;
    else
        vefem::set_global_error(msg);
    return code;
}

#define BCK(call)                                                                          \
    do {                                                                                   \
        cudaError_t _e = (call);                                                           \
        if (_e != cudaSuccess)                                                             \
            return bfail(bt, VEFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

int spec_of(const KParams &p) { return (p.ReN == 0.0 ? SPEC_RE0 : 0) | (p.DfN == 0.0 ? SPEC_DF0 : 0); }

int build_work(vefem_batch *bt)
{
    std::vector<WorkItem> rw, xw;
    for (int i = 0; i < bt->ninst; i++) {
        const int nel = bt->ctx[i]->nel;
        for (int e0 = 0; e0 < nel; e0 += RES_EPB) rw.push_back({i, e0, std::min(RES_EPB, nel - e0), 0});
        const int tile = bt->tiles[size_class(nel)];
        for (int e0 = 0; e0 < nel; e0 += tile) xw.push_back({i, e0, std::min(tile, nel - e0), 0});
    }
    cudaFree(bt->d_res_work);
    cudaFree(bt->d_ex_work);
    bt->d_res_work = bt->d_ex_work = nullptr;
    BCK(cudaMalloc(&bt->d_res_work, rw.size() * sizeof(WorkItem)));
    BCK(cudaMalloc(&bt->d_ex_work, xw.size() * sizeof(WorkItem)));
    BCK(cudaMemcpy(bt->d_res_work, rw.data(), rw.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(bt->d_ex_work, xw.data(), xw.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    bt->n_res_work = (int)rw.size();
    bt->n_ex_work = (int)xw.size();
    if (!bt->d_sc_work) {
        std::vector<ScatterItem> sw;
        for (int i = 0; i < bt->ninst; i++) {
            const vefem_ctx *c = bt->ctx[i];
            const int64_t n6 = (int64_t)c->nnodes * 6, nj = (int64_t)c->nblocks * 36;
            for (int64_t f = 0; f < n6; f += SC_RES_RUN)
                sw.push_back({i, SC_RES, f, (int)std::min<int64_t>(SC_RES_RUN, n6 - f), 0});
            for (int64_t f = 0; f < nj; f += SC_JAC_RUN)
                sw.push_back({i, SC_JAC, f, (int)std::min<int64_t>(SC_JAC_RUN, nj - f), 0});
            if (c->nex) {
                for (int64_t f = 0; f < n6; f += SC_RES_RUN)
                    sw.push_back({i, SC_ARC, f, (int)std::min<int64_t>(SC_RES_RUN, n6 - f), 0});
                const int64_t r0 = c->h_rowptr[n6], r1 = c->h_rowptr[c->N];
                for (int64_t f = r0; f < r1; f += SC_RES_RUN)
                    sw.push_back({i, SC_EXTRA, f, (int)std::min<int64_t>(SC_RES_RUN, r1 - f), 0});
                if (r1 == r0) sw.push_back({i, SC_EXTRA, r0, 0, 0});
            }
        }
        BCK(cudaMalloc(&bt->d_sc_work, sw.size() * sizeof(ScatterItem)));
        BCK(cudaMemcpy(bt->d_sc_work, sw.data(), sw.size() * sizeof(ScatterItem), cudaMemcpyHostToDevice));
        bt->n_sc_work = (int)sw.size();
    }
    if (bt->graph) {
        cudaGraphExecDestroy(bt->graph);
        bt->graph = nullptr;
        bt->key = GraphKey();
    }
    return VEFEM_OK;
}

int ensure_scratch(vefem_batch *bt, size_t elem)
{
    if (!bt->d_rs) BCK(cudaMalloc(&bt->d_rs, (size_t)bt->total_el * 54 * sizeof(double)));
    if (elem && bt->es_elem != elem) {
        cudaFree(bt->d_es);
        cudaFree(bt->d_as);
        bt->d_es = bt->d_as = nullptr;
        BCK(cudaMalloc(&bt->d_es, (size_t)bt->total_el * 2916 * elem));
        BCK(cudaMalloc(&bt->d_as, (size_t)bt->total_el * 54 * elem));
        bt->es_elem = elem;
    }
    return VEFEM_OK;
}

void launch_all(vefem_batch *bt, int flags, bool timing, cudaError_t *err)
{
    cudaStream_t s = bt->s;
    const bool want_res = flags & VEFEM_RESIDUAL;
    const int jmode = flags & (VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32);
    const bool f32 = jmode == VEFEM_JAC_EXACT32;
    const size_t vsize = f32 ? sizeof(float) : sizeof(double);
    cudaError_t e = cudaSuccess;
    bt->launches = 0;
    if (timing && e == cudaSuccess) e = cudaEventRecord(bt->ev[0], s);
    // VEFEM_ZERO_FIRST: the scatter starts its sums from zero (no memsets)
    const int store = (flags & VEFEM_ZERO_FIRST) ? 1 : 0;
    if (timing && e == cudaSuccess) e = cudaEventRecord(bt->ev[1], s);
    const int res_grid = bt->sms * std::max(1, residual_batched_ctas_per_sm(bt->form, bt->spec));
    const int ex_grid = bt->sms * std::max(1, exact_batched_ctas_per_sm((int)vsize, bt->form, bt->spec));
    const bool side = want_res && jmode;
    if (want_res && e == cudaSuccess) {
        cudaStream_t rs = s;
        if (side) {
            e = cudaEventRecord(bt->fork, s);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(bt->s2, bt->fork, 0);
            rs = bt->s2;
        }
        if (e == cudaSuccess)
            e = launch_residual64_batched(bt->d_inst, bt->d_res_work, bt->n_res_work, bt->form,
                                          bt->spec, std::min(res_grid, bt->n_res_work), rs);
        if (side && e == cudaSuccess) e = cudaEventRecord(bt->join, bt->s2);
        bt->launches++;
    }
    if (jmode && e == cudaSuccess) {
        const int g = std::min(ex_grid, bt->n_ex_work);
        e = f32 ? launch_exact_batched<float>(bt->d_inst, bt->d_ex_work, bt->n_ex_work, bt->form,
                                              bt->spec, g, s)
                : launch_exact_batched<double>(bt->d_inst, bt->d_ex_work, bt->n_ex_work, bt->form,
                                               bt->spec, g, s);
        bt->launches++;
    }
    if (side && e == cudaSuccess) e = cudaStreamWaitEvent(s, bt->join, 0);
    if (timing && e == cudaSuccess) e = cudaEventRecord(bt->ev[2], s);
    // scatter: one persistent launch over the scatter work list
    if (e == cudaSuccess) {
        const int grid = std::min(bt->n_sc_work, bt->sms * 8);
        if (f32)
            k_scatter_batched<float><<<grid, SC_THREADS, 0, s>>>(bt->d_inst, bt->d_sc_work, bt->n_sc_work,
                                                                want_res, jmode != 0, store);
        else
            k_scatter_batched<double><<<grid, SC_THREADS, 0, s>>>(bt->d_inst, bt->d_sc_work, bt->n_sc_work,
                                                                 want_res, jmode != 0, store);
        e = cudaGetLastError();
        bt->launches++;
    }
    if (timing && e == cudaSuccess) e = cudaEventRecord(bt->ev[3], s);
    *err = e;
}

}  // namespace

extern "C" int vefem_batch_create(int ninst, const vefem_mesh *meshes, const vefem_csr *patterns,
                                  const vefem_params *params, vefem_batch **out)
{
    vefem_batch *bt = nullptr;
    if (!out || ninst <= 0 || !meshes || !patterns || !params)
        return bfail(nullptr, VEFEM_ERR_ARG, "vefem_batch_create: bad arguments");
    *out = nullptr;
    for (int i = 1; i < ninst; i++) {
        if (params[i].device != params[0].device || params[i].form != params[0].form ||
            params[i].nex != params[0].nex || (params[i].ReN == 0.0) != (params[0].ReN == 0.0) ||
            (params[i].DfN == 0.0) != (params[0].DfN == 0.0))
            return bfail(nullptr, VEFEM_ERR_ARG,
                         "vefem_batch_create: instances differ in device, form, nex or the "
                         "zero pattern of ReN/DfN");
    }
    bt = new vefem_batch();
    bt->ninst = ninst;
    bt->device = params[0].device;
    bt->nex = params[0].nex;
    for (int i = 0; i < ninst; i++) {
        vefem_ctx *c = nullptr;
        int rc = vefem_create(&meshes[i], &patterns[i], &params[i], &c);
        if (rc) {
            std::string m = std::string("vefem_batch_create: instance ") + std::to_string(i) + ": " +
                            vefem_last_error(nullptr);
            vefem_batch_destroy(bt);
            return bfail(nullptr, rc, m);
        }
        bt->ctx.push_back(c);
    }
    bt->form = bt->ctx[0]->prm.form;
    bt->spec = spec_of(bt->ctx[0]->prm);
    auto init = [&]() -> int {
        BCK(cudaSetDevice(bt->device));
        BCK(cudaDeviceGetAttribute(&bt->sms, cudaDevAttrMultiProcessorCount, bt->device));
        BCK(cudaStreamCreateWithFlags(&bt->s, cudaStreamNonBlocking));
        BCK(cudaStreamCreateWithFlags(&bt->s2, cudaStreamNonBlocking));
        BCK(cudaEventCreateWithFlags(&bt->fork, cudaEventDisableTiming));
        BCK(cudaEventCreateWithFlags(&bt->join, cudaEventDisableTiming));
        for (auto &ev : bt->ev) BCK(cudaEventCreate(&ev));
        for (int i = 0; i < ninst; i++) bt->total_el += bt->ctx[i]->nel;
        BCK(cudaMalloc(&bt->d_inst, ninst * sizeof(BatchInst)));
        bt->h_inst.resize(ninst);
        for (int i = 0; i < ninst; i++) {
            BatchInst &I = bt->h_inst[i];
            std::memset(&I, 0, sizeof(I));
            const vefem_ctx *c = bt->ctx[i];
            I.ea.nel = c->nel;
            I.ea.nnodes = c->nnodes;
            I.ea.conn = c->d_conn;
            I.ea.xy = c->d_xy;
            I.prm = c->prm;
            I.ga.nnodes = c->nnodes;
            I.ga.nblocks = c->nblocks;
            I.ga.nex = c->nex;
            I.ga.rowptr = c->d_rowptr;
            I.ga.nptr = c->d_nptr;
            I.ga.ncon = c->d_ncon;
            I.ga.brow = c->d_brow;
            I.ga.boff = c->d_boff;
            I.ga.bptr = c->d_bptr;
            I.ga.bcon = c->d_bcon;
        }
        return build_work(bt);
    };
    if (int rc = init()) {
        std::string m = "vefem_batch_create: " + bt->err;
        vefem_batch_destroy(bt);
        return bfail(nullptr, rc, m);
    }
    *out = bt;
    return VEFEM_OK;
}

extern "C" int vefem_batch_set_params(vefem_batch *bt, int inst, const vefem_params *p)
{
    if (!bt || !p || inst < 0 || inst >= bt->ninst) return bfail(bt, VEFEM_ERR_ARG, "bad instance");
    if (p->form != bt->ctx[0]->prm.form ||
        ((p->ReN == 0.0 ? SPEC_RE0 : 0) | (p->DfN == 0.0 ? SPEC_DF0 : 0)) != bt->spec)
        return bfail(bt, VEFEM_ERR_ARG, "form and the zero pattern of ReN/DfN are fixed at create");
    if (int rc = vefem_set_params(bt->ctx[inst], p))
        return bfail(bt, rc, vefem_last_error(bt->ctx[inst]));
    bt->h_inst[inst].prm = bt->ctx[inst]->prm;
    bt->key = GraphKey();           // descriptors re-uploaded on the next call
    return VEFEM_OK;
}

extern "C" int vefem_assemble_batched(vefem_batch *bt, const double *const *TL,
                                      const double *const *EU, int flags, double *const *b,
                                      void *const *vals, int on_device)
{
    if (!bt) return VEFEM_ERR_ARG;
    const int known = VEFEM_RESIDUAL | VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32 | VEFEM_ZERO_FIRST |
                      VEFEM_TIMING;
    if (flags & (VEFEM_JAC_FD64 | VEFEM_OUTLET_EDGES))
        return bfail(bt, VEFEM_ERR_UNSUPPORTED, "FD64 and outlet edges are not batched");
    if (flags & ~known) return bfail(bt, VEFEM_ERR_UNSUPPORTED, "unknown flag");
    const int jmode = flags & (VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32);
    if (jmode == (VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32))
        return bfail(bt, VEFEM_ERR_ARG, "at most one Jacobian flag");
    const bool want_res = flags & VEFEM_RESIDUAL;
    if (!want_res && !jmode) return bfail(bt, VEFEM_ERR_ARG, "nothing requested");
    if (!TL || (bt->nex && !EU) || (want_res && !b) || (jmode && !vals))
        return bfail(bt, VEFEM_ERR_ARG, "NULL pointer array");
    for (int i = 0; i < bt->ninst; i++)
        if (!TL[i] || (bt->nex && !EU[i]) || (want_res && !b[i]) || (jmode && !vals[i]))
            return bfail(bt, VEFEM_ERR_ARG, "NULL pointer for instance " + std::to_string(i));
    const size_t vsize = jmode == VEFEM_JAC_EXACT32 ? sizeof(float) : sizeof(double);
    const bool timing = flags & VEFEM_TIMING;
    BCK(cudaSetDevice(bt->device));
    if (int rc = ensure_scratch(bt, jmode ? vsize : 0)) return rc;
    cudaStream_t s = bt->s;
    float copy_ms = 0.0f;
    cudaEvent_t c0 = bt->ev[0], c1 = bt->ev[1];

    // device pointers of this call (staging for host buffers)
    std::vector<const double *> dTL(bt->ninst), dEU(bt->ninst);
    std::vector<double *> db(bt->ninst);
    std::vector<void *> dv(bt->ninst);
    if (!on_device) {
        if (bt->st_TL.empty()) {
            bt->st_TL.assign(bt->ninst, nullptr);
            bt->st_EU.assign(bt->ninst, nullptr);
            bt->st_b.assign(bt->ninst, nullptr);
            bt->st_vals.assign(bt->ninst, nullptr);
            for (int i = 0; i < bt->ninst; i++) {
                BCK(cudaMalloc(&bt->st_TL[i], bt->ctx[i]->nnodes * 6 * sizeof(double)));
                BCK(cudaMalloc(&bt->st_EU[i], std::max(1, bt->nex) * sizeof(double)));
                BCK(cudaMalloc(&bt->st_b[i], bt->ctx[i]->N * sizeof(double)));
            }
        }
        if (jmode && bt->st_vals_elem != vsize) {
            for (int i = 0; i < bt->ninst; i++) {
                cudaFree(bt->st_vals[i]);
                BCK(cudaMalloc(&bt->st_vals[i], bt->ctx[i]->nnz * vsize));
            }
            bt->st_vals_elem = vsize;
        }
        if (timing) BCK(cudaEventRecord(c0, s));
        for (int i = 0; i < bt->ninst; i++) {
            const vefem_ctx *c = bt->ctx[i];
            BCK(cudaMemcpyAsync(bt->st_TL[i], TL[i], c->nnodes * 6 * sizeof(double), cudaMemcpyHostToDevice, s));
            if (bt->nex) BCK(cudaMemcpyAsync(bt->st_EU[i], EU[i], bt->nex * sizeof(double), cudaMemcpyHostToDevice, s));
            if (want_res && !(flags & VEFEM_ZERO_FIRST))
                BCK(cudaMemcpyAsync(bt->st_b[i], b[i], c->N * sizeof(double), cudaMemcpyHostToDevice, s));
            if (jmode && !(flags & VEFEM_ZERO_FIRST))
                BCK(cudaMemcpyAsync(bt->st_vals[i], vals[i], c->nnz * vsize, cudaMemcpyHostToDevice, s));
            dTL[i] = bt->st_TL[i];
            dEU[i] = bt->st_EU[i];
            db[i] = bt->st_b[i];
            dv[i] = jmode ? bt->st_vals[i] : nullptr;
        }
        if (timing) {
            BCK(cudaEventRecord(c1, s));
            BCK(cudaEventSynchronize(c1));
            cudaEventElapsedTime(&copy_ms, c0, c1);
        }
    } else {
        for (int i = 0; i < bt->ninst; i++) {
            dTL[i] = TL[i];
            dEU[i] = bt->nex ? EU[i] : nullptr;
            db[i] = want_res ? b[i] : nullptr;
            dv[i] = jmode ? vals[i] : nullptr;
        }
    }
    // descriptors of this call
    GraphKey key;
    key.flags = flags & ~VEFEM_TIMING;
    for (int i = 0; i < bt->ninst; i++) {
        BatchInst &I = bt->h_inst[i];
        I.ea.TL = dTL[i];
        I.ea.EU = dEU[i];
        I.b = db[i];
        I.vals = dv[i];
        key.ptrs.push_back(dTL[i]);
        key.ptrs.push_back(dEU[i]);
        key.ptrs.push_back(db[i]);
        key.ptrs.push_back(dv[i]);
    }
    {
        int64_t e_off = 0;
        for (int i = 0; i < bt->ninst; i++) {
            BatchInst &I = bt->h_inst[i];
            I.ea.rs = bt->d_rs + e_off * 54;
            I.es = jmode ? (void *)((char *)bt->d_es + e_off * 2916 * vsize) : nullptr;
            I.as = jmode ? (void *)((char *)bt->d_as + e_off * 54 * vsize) : nullptr;
            I.ea.es = nullptr;
            I.ea.as = nullptr;
            e_off += bt->ctx[i]->nel;
        }
    }
    const bool same = bt->graph && key == bt->key;
    if (!same) BCK(cudaMemcpyAsync(bt->d_inst, bt->h_inst.data(), bt->ninst * sizeof(BatchInst),
                                   cudaMemcpyHostToDevice, s));
    cudaError_t le = cudaSuccess;
    if (timing) {
        launch_all(bt, flags, true, &le);
        BCK(le);
    } else {
        if (!same) {
            if (bt->graph) cudaGraphExecDestroy(bt->graph);
            bt->graph = nullptr;
            cudaGraph_t g;
            BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            launch_all(bt, flags, false, &le);
            cudaError_t ce = cudaStreamEndCapture(s, &g);
            BCK(le);
            BCK(ce);
            BCK(cudaGraphInstantiate(&bt->graph, g, 0));
            cudaGraphDestroy(g);
            bt->key = key;
        }
        BCK(cudaGraphLaunch(bt->graph, s));
        bt->replays++;
    }
    if (!on_device) {
        for (int i = 0; i < bt->ninst; i++) {
            const vefem_ctx *c = bt->ctx[i];
            if (want_res) BCK(cudaMemcpyAsync(b[i], db[i], c->N * sizeof(double), cudaMemcpyDeviceToHost, s));
            if (jmode) BCK(cudaMemcpyAsync(vals[i], dv[i], c->nnz * vsize, cudaMemcpyDeviceToHost, s));
        }
    }
    BCK(cudaStreamSynchronize(s));
    if (timing) {
        float z = 0, el = 0, ga = 0;
        cudaEventElapsedTime(&z, bt->ev[0], bt->ev[1]);
        cudaEventElapsedTime(&el, bt->ev[1], bt->ev[2]);
        cudaEventElapsedTime(&ga, bt->ev[2], bt->ev[3]);
        bt->timing[0] = el;
        bt->timing[1] = ga;
        bt->timing[2] = z + copy_ms;
    }
    return VEFEM_OK;
}

extern "C" int vefem_batch_set_tiles(vefem_batch *bt, const int *tiles)
{
    if (!bt || !tiles) return bfail(bt, VEFEM_ERR_ARG, "NULL argument");
    for (int c = 0; c < VEFEM_BATCH_CLASSES; c++)
        if (tiles[c] < 1 || tiles[c] > 64) return bfail(bt, VEFEM_ERR_ARG, "tile out of 1..64");
    BCK(cudaSetDevice(bt->device));
    std::memcpy(bt->tiles, tiles, sizeof(bt->tiles));
    return build_work(bt);
}

extern "C" int vefem_batch_autotune(vefem_batch *bt, int flags, int reps, int *tiles_out)
{
    if (!bt || reps <= 0) return bfail(bt, VEFEM_ERR_ARG, "bad arguments");
    const int jmode = flags & (VEFEM_JAC_EXACT64 | VEFEM_JAC_EXACT32);
    if (!jmode || (flags & (VEFEM_JAC_FD64 | VEFEM_OUTLET_EDGES)))
        return bfail(bt, VEFEM_ERR_ARG, "autotune needs an exact Jacobian flag");
    const size_t vsize = jmode == VEFEM_JAC_EXACT32 ? sizeof(float) : sizeof(double);
    BCK(cudaSetDevice(bt->device));
    if (int rc = ensure_scratch(bt, vsize)) return rc;
    // own device inputs: the zero state would divide by zero in the SQRT form,
    // so every instance gets the identity conformation and zero velocity
    std::vector<double *> tl(bt->ninst), eu(bt->ninst);
    for (int i = 0; i < bt->ninst; i++) {
        const int nn = bt->ctx[i]->nnodes;
        std::vector<double> h((size_t)nn * 6, 0.0);
        const bool sqrt_form = bt->form == FORM_SQRT;
        for (int n = 0; n < nn; n++) {
            h[(size_t)3 * nn + n] = sqrt_form ? 1.0 : 0.0;
            h[(size_t)5 * nn + n] = sqrt_form ? 1.0 : 0.0;
        }
        BCK(cudaMalloc(&tl[i], h.size() * sizeof(double)));
        BCK(cudaMemcpy(tl[i], h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        const double one = 1.0;
        BCK(cudaMalloc(&eu[i], sizeof(double)));
        BCK(cudaMemcpy(eu[i], &one, sizeof(double), cudaMemcpyHostToDevice));
    }
    for (int i = 0; i < bt->ninst; i++) {
        BatchInst &I = bt->h_inst[i];
        I.ea.TL = tl[i];
        I.ea.EU = eu[i];
    }
    int64_t e_off = 0;
    for (int i = 0; i < bt->ninst; i++) {
        BatchInst &I = bt->h_inst[i];
        I.es = (char *)bt->d_es + e_off * 2916 * vsize;
        I.as = (char *)bt->d_as + e_off * 54 * vsize;
        e_off += bt->ctx[i]->nel;
    }
    BCK(cudaMemcpy(bt->d_inst, bt->h_inst.data(), bt->ninst * sizeof(BatchInst), cudaMemcpyHostToDevice));
    bt->key = GraphKey();
    const int ex_grid = bt->sms * std::max(1, exact_batched_ctas_per_sm((int)vsize, bt->form, bt->spec));
    int chosen[VEFEM_BATCH_CLASSES];
    std::memcpy(chosen, bt->tiles, sizeof(chosen));
    for (int c = 0; c < VEFEM_BATCH_CLASSES; c++) {
        bool present = false;
        for (int i = 0; i < bt->ninst; i++) present |= size_class(bt->ctx[i]->nel) == c;
        if (!present) continue;
        float best = 1e30f;
        for (int tile : EX_TILES) {
            std::vector<WorkItem> w;
            for (int i = 0; i < bt->ninst; i++) {
                const int nel = bt->ctx[i]->nel;
                if (size_class(nel) != c) continue;
                for (int e0 = 0; e0 < nel; e0 += tile) w.push_back({i, e0, std::min(tile, nel - e0), 0});
            }
            WorkItem *dw = nullptr;
            BCK(cudaMalloc(&dw, w.size() * sizeof(WorkItem)));
            BCK(cudaMemcpy(dw, w.data(), w.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
            const int g = std::min<int>(ex_grid, (int)w.size());
            cudaError_t le = cudaSuccess;
            auto go = [&]() {
                le = vsize == 4 ? launch_exact_batched<float>(bt->d_inst, dw, (int)w.size(), bt->form, bt->spec, g, bt->s)
                                : launch_exact_batched<double>(bt->d_inst, dw, (int)w.size(), bt->form, bt->spec, g, bt->s);
            };
            go();   // warm-up
            BCK(le);
            BCK(cudaEventRecord(bt->ev[0], bt->s));
            for (int r = 0; r < reps; r++) go();
            BCK(le);
            BCK(cudaEventRecord(bt->ev[1], bt->s));
            BCK(cudaEventSynchronize(bt->ev[1]));
            float ms = 0;
            cudaEventElapsedTime(&ms, bt->ev[0], bt->ev[1]);
            cudaFree(dw);
            if (ms < best) {
                best = ms;
                chosen[c] = tile;
            }
        }
    }
    for (int i = 0; i < bt->ninst; i++) {
        cudaFree(tl[i]);
        cudaFree(eu[i]);
    }
    std::memcpy(bt->tiles, chosen, sizeof(chosen));
    if (tiles_out) std::memcpy(tiles_out, chosen, sizeof(chosen));
    return build_work(bt);
}

extern "C" int vefem_batch_info(const vefem_batch *bt, int64_t out[6])
{
    if (!bt || !out) return VEFEM_ERR_ARG;
    out[0] = bt->ninst;
    out[1] = bt->total_el;
    out[2] = bt->n_ex_work;
    const size_t vs = bt->es_elem ? bt->es_elem : sizeof(float);
    out[3] = (int64_t)bt->sms * std::max(1, exact_batched_ctas_per_sm((int)vs, bt->form, bt->spec));
    out[4] = bt->launches;
    out[5] = bt->replays;
    return VEFEM_OK;
}

extern "C" int vefem_batch_last_timing(const vefem_batch *bt, float ms[3])
{
    if (!bt || !ms) return VEFEM_ERR_ARG;
    for (int i = 0; i < 3; i++) ms[i] = bt->timing[i];
    return VEFEM_OK;
}

extern "C" int vefem_batch_destroy(vefem_batch *bt)
{
    if (!bt) return VEFEM_OK;
    cudaSetDevice(bt->device);
    if (bt->s) cudaStreamSynchronize(bt->s);
    if (bt->graph) cudaGraphExecDestroy(bt->graph);
    for (vefem_ctx *c : bt->ctx) vefem_destroy(c);
    void *p[] = {bt->d_inst, bt->d_res_work, bt->d_ex_work, bt->d_sc_work,
                 bt->d_rs, bt->d_es, bt->d_as};
    for (void *q : p)
        if (q) cudaFree(q);
    for (double *q : bt->st_TL) cudaFree(q);
    for (double *q : bt->st_EU) cudaFree(q);
    for (double *q : bt->st_b) cudaFree(q);
    for (void *q : bt->st_vals) cudaFree(q);
    for (auto &ev : bt->ev)
        if (ev) cudaEventDestroy(ev);
    if (bt->s2) cudaStreamSynchronize(bt->s2);
    if (bt->fork) cudaEventDestroy(bt->fork);
    if (bt->join) cudaEventDestroy(bt->join);
    if (bt->s2) cudaStreamDestroy(bt->s2);
    if (bt->s) cudaStreamDestroy(bt->s);
    delete bt;
    return VEFEM_OK;
}

extern "C" const char *vefem_batch_last_error(const vefem_batch *bt) { return bt ? bt->err.c_str() : ""; }
