// batch.h — host-side structures of the batched launch (shared by batch.cu and serve.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "dispatch.h"

namespace stc {

constexpr int kBatchThreads = 256;
constexpr int kBatchMaxL = 128;
constexpr int kBatchMaxR = 8;

// reduction parameters in the form the op structs read (see map_kernel.cuh)
struct OpArgs {
    int32_t L;
    uint32_t birth, survive;
    double alpha;
    float rcp_f;
    int32_t fastdiv_f;
    float Lf;
    double Ld;
    float alpha_f;
    const float* wf;
    const double* w;
};

struct BatchJob {
    void* buf[2];
    int64_t org[2];
    int64_t sy[2];
    int32_t n0, n1;
    int32_t dtype, opv, boundary;
    int32_t L, R;
    int32_t tw, th, k;
    int32_t ntx, nty, tiles;
    int32_t rounds, nsteps;
    int32_t resident;
    int32_t vec;            // tiled with the vector-column map (one step per round, tile 32*XV x 8*VS)
    int32_t shape;          // stc_shape when the job's table is that generated shape (radius R), else 0
    int32_t counter_base, off_base;
    float padf;
    int32_t padi;
    double alpha;
    uint32_t birth, survive;
    float rcp_f;
    int32_t fastdiv_f;
};

struct BatchItem { int32_t job, round, tile, steps; };

struct BatchDev {
    const BatchJob* jobs;
    const BatchItem* items;
    int nitems;
    int* ticket;
    int* counters;
    int* abort_flag;
    int* status;
    const int8_t* offs;   // 2 per offset
    const float* wts;
};

struct BatchSpec {
    stc_grid a, b;
    std::vector<int32_t> offs;   // (x, y) pairs
    std::vector<double> wts;
    int L = 0, R = 0, wdt = STC_F64, shape = STC_SHAPE_TABLE;
    stc_op op{};
    stc_bc bc{};
    int64_t nsteps = 0;
    int opv = 0;
    int force_tw = 0, force_th = 0, force_k = 0;   // autotuner trials: k-step tiles of this geometry
    int force_vec = 0;                              // autotuner trials: one-step vector-column tiles
};

// tiled-job geometry; vec = 1 selects one-step vector-column tiles (tw, th fixed by the element type)
struct Geometry { int tw, th, k; int vec = 0; };

}  // namespace stc

struct stc_batch {
    std::vector<stc::BatchSpec> specs;
    std::vector<stc::BatchJob> hjobs;
    std::vector<stc::BatchItem> hitems;
    std::vector<int8_t> hoffs;
    std::vector<float> hwts;
    std::vector<int> result_in_b;
    int ncounters = 0;
    void* dmem = nullptr;
    size_t dmem_bytes = 0;
    stc::BatchDev dev{};
    stc::StatusSlot slot{};   // this batch's timeout word, baked into the planned launch
    size_t smem = 0;
    int grid = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool planned = false;
    bool prefer_vec = false;   // plan vector tiles wherever the shape has them, ignoring tuned geometries
    double planned_cell_steps = 0;
};

namespace stc {
// Plan jobs, upload tables and capture (counter reset + kernel) as a CUDA graph (capture = true), or
// only prepare a direct launch (capture = false, see batch_launch).
int batch_build(stc_batch* b, bool autotune, cudaStream_t stream, DeviceCtx* ctx, bool capture = true);
// Reset counters and launch the planned queue directly on `stream` (no graph).
int batch_launch(stc_batch* b, cudaStream_t stream);
void batch_free(stc_batch* b);
}  // namespace stc
