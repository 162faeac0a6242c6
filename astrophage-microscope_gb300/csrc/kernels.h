// kernels.h -- host-side launchers of the engine's kernels (one per stage
// piece). Every launcher enqueues on the given stream and never synchronises.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "dev.cuh"

namespace agb {

struct WorldConst;   // defined in world.cuh

// Fields (k_grid.cu)
void launch_fill(float* v, int64_t n, float value, cudaStream_t s);
// The brush disc over columns [x0, x0 + bw) x [y0, y0 + bh) of every plane.
void launch_brush(float* v, const GridDev& g, float cx, float cy, float radius, float amount,
                  int32_t x0, int32_t y0, int32_t bw, int32_t bh, cudaStream_t s);
// Tiling of the TMA stencil for a grid: lanes along x (16 or 32), rows per
// thread (1, 2, 4) and z planes per CTA. A tensor map's box is made for one
// tiling and is used only with it.
struct FtcsPlan { int32_t lx, rpt, zc; };
FtcsPlan ftcs_plan(int32_t nx, int32_t ny, int32_t nz);
// A given tiling (lx 16/32, rpt 1/2/4; lx 16 with rpt 4 is not built) with the
// z chunk chosen as ftcs_plan chooses it when zc <= 0.
FtcsPlan ftcs_plan_with(int32_t nx, int32_t ny, int32_t nz, int32_t lx, int32_t rpt, int32_t zc);
// The same for `copies` grids in one launch (batched passes): the z chunk fills
// one wave with all of them.
FtcsPlan ftcs_plan_copies(int32_t nx, int32_t ny, int32_t nz, int32_t lx, int32_t rpt, int32_t zc,
                          int32_t copies);
// One explicit FTCS pass src -> dst (src/fields/diffuse.cu:19-44; 7-point when nz > 1).
// 3-D grids with a tensor map (and the tiling it was made for) use the TMA-staged kernel.
// Returns the launch's status.
cudaError_t launch_ftcs(const GridDev& g, const float* src, float* dst, float coeff, const int32_t* bc,
                        const float* face, float robin, const CUtensorMap* src_map, const FtcsPlan* plan,
                        uint32_t* err, cudaStream_t s);
// Whether the plain FTCS kernels (the path without a tensor map) can be
// launched on this grid: their launch grids have at most 65535 blocks along y
// (8 rows each) and along z (8 planes each).
bool ftcs_plain_fits(int32_t nx, int32_t ny, int32_t nz);
bool make_plane_map(CUtensorMap* map, float* base, int32_t nx, int32_t ny, int32_t nz, const FtcsPlan& plan);
// One chamber's FTCS pass in a batched launch (agb_batch). The chambers of a
// launch share grid dimensions and tiling; each has its own tensor map (over
// the pass's source buffer, made for that tiling), destination and faces.
struct FtcsChamber {
    CUtensorMap map;
    float* dst;
    uint32_t* err;
    float coeff, robin;
    int32_t bc[6];
    float face[6];
};
void launch_ftcs_batch(const FtcsChamber* tab, int32_t nch, int32_t nx, int32_t ny, int32_t nz,
                       const FtcsPlan& plan, cudaStream_t s);
// Fold deposits into the field for the voxels cells sit in (flush_kernel,
// src/fields/diffuse.cu:51-60, restricted to voxels that can hold a deposit).
// `temperature`: the temperature grid's flush, skipped on the device when no
// thermal substep has deposited heat since the previous one.
// `vox`: each cell's voxel in g when known (the thermal substeps' record), else null.
void launch_flush_by_cells(DevState* S, GridDev g, unsigned long long* demand_to_clear,
                           int32_t grid_blocks, cudaStream_t s, bool temperature, const int32_t* vox);

// Spatial hash (k_hash.cu)
void hash_build(DevState* S, const HashDev& h, int32_t capacity, uint32_t* sort_keys_alt,
                uint32_t* sort_vals_alt, uint32_t* hist, int32_t grid_blocks, cudaStream_t s);
// 32-bit words of sort scratch (`hist`) hash_build needs at this capacity.
size_t hash_sort_scratch_words(int32_t capacity);

}  // namespace agb
