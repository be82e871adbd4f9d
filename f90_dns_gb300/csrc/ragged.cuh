// Ragged multi-run launches: one kernel launch advances one stage of the time
// step for many independent runs whose grids (nx, ny, nz) differ.
//
// Every run has a descriptor (RunDesc: its grid constants, operators and
// buffer pointers) in device memory.  A stage's launch covers the "virtual
// blocks" of all runs -- a virtual block is what the stage's single-run kernel
// does in one CTA (one mode tile, one group of transform columns, one slice of
// an elementwise pass) -- and run order[i] owns virtual blocks
// [start[i], start[i+1]).  A CTA finds its run by binary search over start,
// copies the run's descriptor into shared memory and executes the single-run
// kernel's body for the local block index, so every run's arithmetic is
// exactly that of its own launches (bitwise the same results).  The grid has
// one CTA per virtual block: the hardware block scheduler balances the
// uneven blocks, and a CTA that strode over several virtual blocks would hold
// the loop's state in registers the bodies need.
#pragma once

#include "dns3d_internal.cuh"

namespace dns3d {

// Stages of one ragged time step, in launch order.
enum RaggedStage {
    kRsVort = 0,  // block 0: PI update; then vorticity mode tiles
    kRsFftYInv,   // inverse y pass of u, v, w, ox, oy, oz
    kRsFftC2R,    // c2r x pass of the same six fields
    kRsProd,      // u x omega in physical space
    kRsFftR2C,    // r2c x pass of the three products
    kRsFftYFwd,   // forward y pass of the products (2/3-filtered columns only)
    kRsVisc,      // viscous step (mixed: the FP32 mode tiles)
    kRsPres,      // pressure solve (mixed: the FP32 mode tiles)
    kRsCorr,      // projection (zero wall planes of u, v, w) and wall gradients of p
    // mixed form only: the FP64 mode (0,0) of the viscous step, then its pinned
    // Poisson solve and dphi/dz, one CTA per run, on a forked stream beside
    // kRsVisc and kRsPres (mode (0,0) of w* is all the pinned solve reads)
    kRsViscMean,
    kRsPresMean,
    // FP64 runs with the tensor-core pressure: the divergence right-hand side
    // (D1.w* on the tensor cores) into PHI, before kRsPres solves it in place
    kRsPresRhs,
    kRsStages
};

// Everything the stage bodies of one run read: copied to shared memory by
// each CTA, so it holds values and pointers only.
struct RunDesc {
    GridDev g;       // g.tc[] holds the tile widths this batch uses
    Ops ops;
    MixedOps mx;
    StepParams sp;
    PIParams pp;
    dns3d_pi_state* pi;
    double2 *U, *V, *W, *P, *GP, *US, *VS, *WS, *PHI, *PHIZ;
    void* spec[6];   // c2r inputs: u, v, w, ox, oy, oz spectra (FP32 or FP64)
    void* tmp[6];    // y-pass outputs
    void* phys[6];   // physical planes; the products overwrite the first three
    void* src[3];    // nonlinear source spectra
    const void* tw_ny;
    const void* tw_nx2;
    const void* tw_nx;
    int* tcerr;              // tensor-core wait status of the run (viscous stage)
    int ncol;                // columns the forward y pass completes
    int gx[kRsStages];       // virtual blocks per field of each stage (transforms, elementwise passes);
                             // kRsVisc: operator indices per CTA of the tensor-core viscous body
    int tcmask;              // z-derivatives on the tensor cores: 1 vorticity, 2 projection, 4 pressure
    int fftfx;               // FP64 transforms in fixed point (twiddles: the Q62 tables)
    int vort_chunk, corr_chunk;  // mode tiles per CTA of those bodies
};

// Work map of one stage launch (device arrays).
struct StageMap {
    const int* start;  // [nruns + 1]; start[nruns] = virtual blocks of the launch
    const int* order;  // [nruns] run index of each slot, largest work first
    int nruns;
};

constexpr int kStageThreads = 256;

// The run slot owning virtual block b: the largest i with start[i] <= b.
__device__ __forceinline__ int stage_slot(const StageMap& map, int b) {
    int lo = 0, hi = map.nruns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&map.start[mid]) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One stage over all runs, one CTA per virtual block.  Stage::run(desc, b) is the single-run
// kernel body; it may use dynamic shared memory (sized by the host to the
// largest run's need) and its own static shared buffers.  Stage::kMinCtas
// bounds the registers so that the stage keeps the occupancy of the
// single-run kernel (descriptor fields held in registers would otherwise
// crowd it out).
template <class Stage>
__global__ void __launch_bounds__(kStageThreads, Stage::kMinCtas)
    k_stage(const RunDesc* __restrict__ runs, StageMap map) {
    __shared__ __align__(16) unsigned char draw[sizeof(RunDesc)];
    const RunDesc& d = *reinterpret_cast<const RunDesc*>(draw);
    const int i = stage_slot(map, blockIdx.x);
    {
        const unsigned long long* s = reinterpret_cast<const unsigned long long*>(runs + __ldg(&map.order[i]));
        unsigned long long* t = reinterpret_cast<unsigned long long*>(draw);
        for (int w = threadIdx.x; w < (int)(sizeof(RunDesc) / 8); w += blockDim.x) t[w] = __ldg(&s[w]);
    }
    __syncthreads();
    Stage::run(d, blockIdx.x - __ldg(&map.start[i]));
}

static_assert(sizeof(RunDesc) % 8 == 0, "descriptor copied in 8-byte words");

// ---------------------------------------------------------------- host side
using StageKernel = void (*)(const RunDesc*, StageMap);

// Kernel variants of FP64 runs: which stages run their tensor-core bodies.
enum RaggedVariant { kRvVortTc = 1, kRvCorrTc = 2, kRvViscTc = 4, kRvPresTc = 8, kRvFftFx = 16 };
int ragged_variant(const RunDesc& d);
// The k_stage instantiation of a stage for FP64 (mixed = false, with the
// variant) or mixed runs (step.cu; the transform passes come from fft_ct.cu).
StageKernel ragged_kernel(int stage, bool mixed, int variant);
StageKernel ragged_fft_kernel(int stage, bool mixed, bool fx);
// CTA columns (y pass) or rows (x passes) of the compile-time transform of length n.
int fft_ct_per_cta(int n);
// Fills d.gx for the run's grid (d.g, d.ncol set).
void ragged_geometry(RunDesc& d);
// Virtual blocks and dynamic shared memory of one run in a stage, with the
// tile widths in d.g.tc.
int ragged_blocks(int stage, bool mixed, const RunDesc& d);
size_t ragged_smem(int stage, bool mixed, const RunDesc& d);
// Whether a stage has a tile width (the mode-tile kernel it uses, or -1).
int ragged_tile_kernel(int stage, bool mixed);

}  // namespace dns3d
