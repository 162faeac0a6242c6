// world_impl.cuh -- the world object behind the C ABI, shared by world.cu
// (one chamber) and batch.cu (many chambers in one graph).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "cells.h"

using namespace agb;   // internal header: the engine's own types

struct GraphEntry {
    int32_t ticks;
    uint32_t parity;        // which buffer holds each field at capture start
    uint64_t tick_phase;    // tick % compaction_period at capture start
    cudaGraphExec_t exec;
    uint32_t parity_after;
    int32_t kernels;        // kernel nodes per replay
};

struct agb_world {
    agb_world_desc d{};
    int dev = 0;
    int sm_count = 0;
    Ctx c{};
    TickParams tp{};
    DevState* S = nullptr;
    void* blob[2] = {nullptr, nullptr};
    size_t blob_bytes = 0;
    float* gbuf[AGB_FIELD_COUNT][2] = {};
    CUtensorMap tmap[AGB_FIELD_COUNT][2];      // TMA maps of each field buffer (3-D grids)
    bool tmap_ok[AGB_FIELD_COUNT] = {};
    FtcsPlan tplan[AGB_FIELD_COUNT] = {};      // the tiling each field's maps were made for
    bool use_tma = true;
    int gcur[AGB_FIELD_COUNT] = {};
    unsigned long long* gdep[AGB_FIELD_COUNT] = {};
    int32_t gbc[AGB_FIELD_COUNT][6] = {};
    float gface[AGB_FIELD_COUNT][6] = {};
    float grobin[AGB_FIELD_COUNT] = {};
    uint32_t *kalt = nullptr, *valt = nullptr, *hist = nullptr;
    LifeBuffers life{};
    int32_t* stamp_idx = nullptr;
    double* occl_factor = nullptr;       // per irradiance voxel: transmittance of stamped voxels
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};   // concurrent branches of a tick
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // Section timers (agb_world_set_timing): a start and an end event per
    // section of the tick, recorded into the captured graph as event nodes.
    bool timing = false;
    cudaEvent_t tev[2 * AGB_TICK_SECTIONS] = {};
    float *fx = nullptr, *fy = nullptr, *fz = nullptr;
    unsigned long long* acc = nullptr;
    int32_t blocks = 1;
    int walk_lanes = 1;                  // threads sharing one cell's neighbour walk (1, 2, 4, 8)
    bool fuse_cells = false;             // feeding, taxis and forces in one kernel with one walk
    // The predator store (k_tau.cu): device state, two blobs (compaction
    // target), per-cell claim words, per-world constants; tau_active once
    // predators have been placed (the tick then runs the predation stage).
    TauState* tS = nullptr;
    void* tau_blob[2] = {nullptr, nullptr};
    int32_t tau_cap = 0;
    unsigned long long* claim = nullptr;
    TauParams taup{};
    bool tau_active = false;
    bool flash_active = false;           // spin-drive flash armed: the flash stage replaces taxis
    double flash_power = AGB_PETROVA_FLASH_POWER;
    unsigned long long* flash_accum = nullptr;   // imp_x, imp_y, imp_z, energy (fixed point)
    int64_t irr_mark_bytes = 0;          // size of c.irr_marks (irradiance lines over any light axis)
    int64_t irr_bit_words = 0;           // size of c.irr_stamp_bits in 32-bit words
    uint64_t tick = 0;
    double sim_time = 0.0;
    double physics_rate = 1.0, biology_rate = 1.0;
    int64_t deaths_reported = 0;
    unsigned long long acc_host[12] = {};
    std::vector<GraphEntry> graphs;
    cudaStream_t own_stream = nullptr;   // capture stream when the caller passes the default stream
    int64_t graph_kernels_total = 0;     // kernel nodes launched by graph replays so far
    uint64_t version = 0;                // bumped whenever captured graphs go stale
    int64_t* xfer_host = nullptr;        // pinned {count, next_id} written by the export kernel
    const void* direct_ptrs[25] = {};    // host arrays last checked as device-accessible
    bool direct_ok = false;
    agb_surrogate* sg = nullptr;         // learned field surrogate driving T and CO2, if attached
    int32_t sg_steps = 0;
    float* sg_q = nullptr;               // per-step heat source of the current window (K)
    std::string err;
    std::vector<void*> allocs;
};

namespace agb {

// One tick of one world enqueued on s (forks onto the world's side streams
// and joins back); advances the host-side tick state as it goes.
void world_tick(agb_world* w, cudaStream_t s);
// Which ping-pong buffer holds each field (bit f = field f), and setting it.
uint32_t world_parity(const agb_world* w);
void world_set_parity(agb_world* w, uint32_t bits);
// tick % compaction period: which compaction decision the next tick takes.
uint64_t world_phase(const agb_world* w);
// Point the context's field views at the current ping-pong buffers.
void world_refresh(agb_world* w);
// Whether this tick runs the irradiance field and feeding; whether the next
// lifecycle stage may compact.
bool world_emission_active(const agb_world* w);
bool world_compaction_allowed(const agb_world* w);
void world_advance_clock(agb_world* w, int32_t ticks);
// Set the tick counter and simulated time (snapshot restore); drops graphs.
void world_set_clock_state(agb_world* w, uint64_t tick, double sim_time);
// Switch field f's stencil tiling (rebuilds its tensor maps); false when the
// field has no TMA path or the maps cannot be made.
bool world_set_tiling(agb_world* w, int f, const FtcsPlan& p);
// Milliseconds per FTCS pass of field f, from a captured graph of 2 * passes
// passes (best of three timed replays). Changes the field's contents.
float world_time_passes(agb_world* w, int f, int passes, cudaStream_t s);

// The surrogate's grid, FTCS steps per call and per-step coefficients (T, CO2).
bool surrogate_info(const agb_surrogate* sg, int32_t dims[3], int32_t* steps, float coeff[2], int32_t bc[2][6]);
// q[i] = deposit[i] / scale / steps (FP32), deposit[i] = 0, for every voxel.
void surrogate_source_from_deposit(unsigned long long* dep, float* q, int64_t n, double inv_scale, int32_t steps,
                                   cudaStream_t s);
// x[i] += q[i].
void surrogate_add(float* x, const float* q, int64_t n, cudaStream_t s);

}  // namespace agb
