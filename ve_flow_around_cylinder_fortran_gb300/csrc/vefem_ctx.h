// Library context of one mesh (internal; the public type is opaque).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "vefem_internal.h"

struct vefem_ctx {
    int device = 0;
    int nnodes = 0, nel = 0, nex = 0;
    int64_t N = 0, nnz = 0;
    int nblocks = 0;
    int nedge = 0;
    int64_t node_nnz = 0;       // AIJ entries of the node rows (rowptr[6 nnodes])
    bool blocks_cover = false;  // element blocks + arclength column = every node-row entry
    vefem::KParams prm{};
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;          // FP64 residual beside an exact Jacobian
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t ev[8] = {};
    float timing[5] = {0, 0, 0, 0, 0};
    int launches = 0;
    std::string err;
    // device tables
    int32_t *d_conn = nullptr;
    double *d_xy = nullptr;
    int64_t *d_rowptr = nullptr;
    int32_t *d_nptr = nullptr, *d_ncon = nullptr;
    int32_t *d_brow = nullptr, *d_boff = nullptr, *d_bptr = nullptr, *d_bcon = nullptr;
    int32_t *d_edge_elem = nullptr, *d_edge_id = nullptr;
    int32_t *d_edge_row = nullptr, *d_edge_off = nullptr;   // [nedge][81]
    int32_t *d_colind = nullptr;                            // for MatZeroRows on the device
    std::vector<int64_t> h_rowptr;                          // host copies for host-side rows
    std::vector<int32_t> h_colind;
    // device scratch / staging (allocated on first use)
    double *d_rs = nullptr, *d_es = nullptr, *d_as = nullptr;
    float *d_es32 = nullptr, *d_as32 = nullptr;
    float *d_vals32 = nullptr;
    double *d_ers = nullptr, *d_ees = nullptr, *d_eas = nullptr;
    double *d_TL = nullptr, *d_EU = nullptr, *d_b = nullptr, *d_vals = nullptr;
    // exact-Jacobian launches go through the batched kernel with this mesh as
    // the only instance (one kernel, so single and batched results agree bit
    // for bit): its descriptor and one work item per element
    vefem::BatchInst h_self{};
    vefem::BatchInst *d_self = nullptr;
    vefem::WorkItem *d_work = nullptr;
    int sms = 0;
    // linear-stability assembly (10 unknowns per node): pattern and scratch
    std::vector<int64_t> h_rowptr10;
    std::vector<int32_t> h_colind10;
    int64_t *d_rowptr10 = nullptr;
    int32_t *d_boff10 = nullptr;
    double *d_ses = nullptr, *d_tlb = nullptr, *d_kw = nullptr;
    double **d_Aptr = nullptr;
    double *d_Astage = nullptr, *d_Bstage = nullptr;
    int stab_nk = 0, stab_nk_stage = 0;
};
