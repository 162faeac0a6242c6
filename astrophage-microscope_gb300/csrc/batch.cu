// batch.cu -- an ensemble of independent chambers advanced by one graph launch.
//
// The reference runs one World per process (src/sim/step.cu:109-184). Here a
// batch owns N complete worlds of uneven cell counts and grid sizes. One call
// to agb_batch_step replays one CUDA graph holding every chamber's tick(s):
// the chambers are spread over `lanes` concurrent branches, heaviest first
// onto the least-loaded branch, and each chamber's tick keeps its own inner
// branches (thermal | hash | slow fields). Small chambers, which alone would
// leave most SMs idle, overlap with the large ones.
//
// The autotuner groups chambers into size classes (temperature grid edge x
// decade of cell count). For each class it builds probe chambers from the
// class's median member and times, with CUDA events, whole graph-replayed
// ticks for every candidate hash cell size, then FTCS passes on the class's
// grids for every stencil tiling; the real chambers are built with the
// winners. A tiling never changes results (every tiling computes each voxel
// with the same operations); the hash cell size changes the order in which
// contacts are summed, so a tuned chamber equals, bit for bit, a standalone
// world built with the hash cell size the tuner picked (agb_batch_tuning).
//
// Staged ticks (the default when every chamber allows them): instead of each
// chamber launching its own ~20 kernels per tick, each stage of the tick is
// one launch over every chamber. The per-world kernel bodies run unchanged;
// a block finds its chamber and its block within that chamber in a block map
// and the chamber's arguments in a table, both in device memory owned by the
// captured graph. FTCS passes are one launch per group of chambers with equal
// grids and tiling, each with its own tensor map. The stages keep the tick's
// order and branches (thermal + irradiance | slow fields | hash), so every
// chamber computes what its own tick would with the same walk shape.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "world_impl.cuh"

namespace {

struct BatchGraph {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec;
    std::vector<uint32_t> parity_after;
    int32_t kernels;
    char* arena;                            // staged graphs: their argument tables and block maps
};

}  // namespace

struct agb_batch {
    std::vector<agb_world*> worlds;
    std::vector<agb_tuning> tuning;
    std::vector<int32_t> order;             // capture order: grouped by lane
    int32_t lanes = 1;
    std::vector<cudaStream_t> lane_streams;
    std::vector<cudaEvent_t> lane_join;
    cudaEvent_t fork = nullptr;
    cudaStream_t own_stream = nullptr;
    bool staged = false;                    // one launch per stage over every chamber
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t sev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    std::vector<BatchGraph> graphs;
    int64_t graph_kernels_total = 0;
    std::string err;
};

namespace {

agb_status bfail(agb_batch* b, agb_status s, const std::string& what) {
    if (b) b->err = what;
    return s;
}

// Bytes one tick moves, for load balancing: cells x 200 B plus 8 B per voxel
// pass of each diffused field.
double tick_bytes(const agb_world_desc& d, int32_t cells) {
    double bytes = 200.0 * cells;
    const double dt = AGB_DT_PHYSICS * (d.physics_rate > 0.0 ? d.physics_rate : 1.0);
    for (int f = 0; f < 3; ++f) {
        const agb_grid_desc& g = d.grid[f];
        if (g.nx <= 0) continue;
        const double vox = (double)g.nx * g.ny * g.nz;
        const double dx = d.chamber_w / g.nx;
        const double lim = g.nz > 1 ? 6.0 : 4.0;
        const double steps = std::floor(dt / (dx * dx / (lim * g.diffusivity))) + 1.0;
        bytes += 8.0 * vox * steps;
    }
    return bytes;
}

std::vector<uint64_t> batch_key(const agb_batch* b, int32_t ticks) {
    std::vector<uint64_t> k;
    k.reserve(b->worlds.size() + 1);
    k.push_back((uint64_t)ticks);
    for (const agb_world* w : b->worlds)
        k.push_back((uint64_t)world_parity(w) | (world_phase(w) << 8) | (w->version << 32));
    return k;
}

void drop_graphs(agb_batch* b) {
    for (auto& g : b->graphs) {
        cudaGraphExecDestroy(g.exec);
        if (g.arena) cudaFree(g.arena);
    }
    b->graphs.clear();
}

// ---------------------------------------------------------------------------
// Staged ticks. plan_tick walks every chamber through one tick in tick_once's
// order, advancing each chamber's host-side state (buffer parities, clock) as
// tick_once does, and records the launches with their tables; run_plan
// replays the recording on the streams (under capture).
// ---------------------------------------------------------------------------
enum class OpKind { Launch, Ftcs, Record, Wait };

struct StagedOp {
    OpKind kind;
    int32_t stream;                         // 0: the step's stream; 1-3: the batch's side streams
    BStage st;
    size_t tab, map;                        // offsets into the arena
    int32_t blocks, arg;
    int32_t nch, nx, ny, nz;
    FtcsPlan plan;
    int32_t event;
};

struct StagedPlan {
    std::vector<char> bytes;
    std::vector<StagedOp> ops;
    std::map<std::vector<uint32_t>, size_t> maps;   // each distinct block map is stored once

    size_t put(const void* p, size_t n) {
        const size_t off = (bytes.size() + 127) & ~(size_t)127;
        bytes.resize(off + n);
        std::memcpy(bytes.data() + off, p, n);
        return off;
    }
    void record(int32_t stream, int32_t ev) {
        StagedOp o{};
        o.kind = OpKind::Record; o.stream = stream; o.event = ev;
        ops.push_back(o);
    }
    void wait(int32_t stream, int32_t ev) {
        StagedOp o{};
        o.kind = OpKind::Wait; o.stream = stream; o.event = ev;
        ops.push_back(o);
    }
    // One batched stage over the chambers of `args` (each with its nblk). The
    // light per-cell stages (a few loads and stores per cell) take half the
    // blocks again: 3.11 -> 3.07 ms per batch64 step.
    void stage(int32_t stream, BStage st, const std::vector<ChamberArgs>& args_in, int32_t arg = 0) {
        std::vector<ChamberArgs> args = args_in;
        switch (st) {
            case BStage::Thermal: case BStage::Flush: case BStage::ClearStamps: case BStage::Stamp:
            case BStage::Occlusion: case BStage::KeyHist: case BStage::Ranges: case BStage::Keep:
            case BStage::ScatterSrc: case BStage::Gather:
                for (ChamberArgs& a : args) a.nblk = std::max(1, (a.nblk + 1) / 2);
                break;
            default: break;
        }
        std::vector<uint32_t> map;
        for (size_t k = 0; k < args.size(); ++k)
            for (int32_t x = 0; x < args[k].nblk; ++x) map.push_back(((uint32_t)k << 16) | (uint32_t)x);
        if (map.empty()) return;
        StagedOp o{};
        o.kind = OpKind::Launch; o.stream = stream; o.st = st; o.arg = arg;
        o.blocks = (int32_t)map.size();
        o.tab = put(args.data(), args.size() * sizeof(ChamberArgs));
        auto it = maps.find(map);
        if (it == maps.end()) it = maps.emplace(map, put(map.data(), map.size() * sizeof(uint32_t))).first;
        o.map = it->second;
        ops.push_back(o);
    }
};

ChamberArgs chamber_args(agb_world* w) {
    world_refresh(w);
    ChamberArgs a{};
    a.S = w->S;
    a.c = w->c;
    a.p = w->tp;
    a.stamp_idx = w->stamp_idx;
    a.factor = w->occl_factor;
    a.fx = w->fx; a.fy = w->fy; a.fz = w->fz;
    a.life = w->life;
    a.kalt = w->kalt; a.valt = w->valt; a.hist = w->hist;
    // A quarter of the blocks a world launches on its own: a world sizes its
    // grid by capacity (twice the cells here), and a batched block first
    // looks up its chamber and that chamber's arguments in global memory, a
    // cost that longer grid-stride loops spread over more cells (per step:
    // 3.50 ms with every block, 3.15 with a quarter, 3.22 with an eighth).
    a.nblk = std::max(1, (w->blocks + 3) / 4);
    const GridDev& co2 = w->c.g[AGB_FIELD_CO2];
    a.demand = co2.enabled ? w->life.co2_demand : nullptr;
    a.gv = co2.enabled ? co2.dx * co2.dx * co2.dz_eff : 0.0;
    bool per4 = true;
    hash_sort_shape(w->c.h, w->c.capacity, a.passes, a.max_tiles, per4, a.radix_bits);
    return a;
}

// One FTCS pass of field f for each chamber of `ws`, grouped by grid and
// tiling; flips each chamber's buffer parity as ftcs() does.
void plan_ftcs(StagedPlan& P, int32_t stream, const std::vector<agb_world*>& ws, int f) {
    std::map<std::vector<int32_t>, std::vector<FtcsChamber>> groups;
    for (agb_world* w : ws) {
        world_refresh(w);
        const GridDev& g = w->c.g[f];
        const FtcsPlan& pl = w->tplan[f];
        FtcsChamber e{};
        e.map = w->tmap[f][w->gcur[f]];
        e.dst = w->gbuf[f][1 - w->gcur[f]];
        e.err = &w->S->error;
        e.coeff = f == AGB_FIELD_TEMPERATURE ? w->tp.t_coeff : (f == AGB_FIELD_CO2 ? w->tp.c_coeff : w->tp.n_coeff);
        e.robin = w->grobin[f];
        for (int k = 0; k < 6; ++k) { e.bc[k] = w->gbc[f][k]; e.face[k] = w->gface[f][k]; }
        groups[{g.nx, g.ny, g.nz, pl.lx, pl.rpt}].push_back(e);
        w->gcur[f] = 1 - w->gcur[f];
        world_refresh(w);
    }
    for (const auto& kv : groups) {
        StagedOp o{};
        o.kind = OpKind::Ftcs; o.stream = stream;
        o.nx = kv.first[0]; o.ny = kv.first[1]; o.nz = kv.first[2];
        o.nch = (int32_t)kv.second.size();
        // Tilings give the same bits; the z chunk is re-chosen for the group.
        o.plan = ftcs_plan_copies(o.nx, o.ny, o.nz, kv.first[3], kv.first[4], 0, o.nch);
        o.tab = P.put(kv.second.data(), kv.second.size() * sizeof(FtcsChamber));
        P.ops.push_back(o);
    }
}

// Whether every chamber can run staged ticks: every diffused grid 3-D with a
// TMA stencil, no surrogate, no spin-drive flash armed, no predators, one lane per cell in
// fused walks, and at most 65,535 blocks per stage (capacities up to about 67M
// cells). Checked at each capture; the lanes path takes the rest.
bool staged_ok(const agb_batch* b) {
    for (const agb_world* w : b->worlds) {
        if (w->sg || w->walk_lanes != 1 || !w->fuse_cells || w->flash_active || w->tau_active) return false;
        // A block map entry holds a chamber's block index in 16 bits.
        if (scan_blocks(w->c.capacity) > 0xFFFF || w->blocks > 0xFFFF) return false;
        for (int f = 0; f < 3; ++f) {
            const GridDev& g = w->c.g[f];
            if (g.enabled && (g.nz <= 1 || !w->use_tma || !w->tmap_ok[f])) return false;
        }
    }
    return true;
}

// tick_once (world.cu) for every chamber at once.
void plan_tick(agb_batch* b, StagedPlan& P) {
    const std::vector<agb_world*>& W = b->worlds;
    const size_t n = W.size();
    P.record(0, 0);
    P.wait(1, 0);
    P.wait(2, 0);
    P.wait(3, 0);
    // Branch 1: thermal substeps, then the irradiance field. A chamber's last
    // substep's flush and FTCS pass fork onto branch 3 once its thermal
    // kernel has run (as in tick_once), beside the irradiance field; earlier
    // substeps' stay on branch 1, ahead of the next thermal kernel.
    std::vector<int32_t> nsub(n, 0);
    int32_t maxsub = 0;
    for (size_t i = 0; i < n; ++i) {
        const agb_world* w = W[i];
        nsub[i] = (w->d.thermal_enabled && w->c.g[AGB_FIELD_TEMPERATURE].enabled) ? w->tp.t_substeps : 0;
        maxsub = std::max(maxsub, nsub[i]);
    }
    for (int32_t k = 0; k < maxsub; ++k) {
        std::vector<agb_world*> mid, fin;
        std::vector<ChamberArgs> th, flm, flf;
        for (size_t i = 0; i < n; ++i) {
            if (k >= nsub[i]) continue;
            ChamberArgs a = chamber_args(W[i]);
            a.arg = k == 0 ? 1 : 0;                      // the first substep records the cells' voxels
            th.push_back(a);
            a.g = W[i]->c.g[AGB_FIELD_TEMPERATURE];
            const bool last = k + 1 == nsub[i];
            (last ? flf : flm).push_back(a);
            (last ? fin : mid).push_back(W[i]);
        }
        P.stage(1, BStage::Thermal, th);
        if (!fin.empty()) {
            P.record(1, 3);
            P.wait(3, 3);
            P.stage(3, BStage::Flush, flf);
            plan_ftcs(P, 3, fin, AGB_FIELD_TEMPERATURE);
        }
        P.stage(1, BStage::Flush, flm);
        plan_ftcs(P, 1, mid, AGB_FIELD_TEMPERATURE);
    }
    P.record(3, 4);
    std::vector<uint8_t> emit(n, 0);
    {
        std::vector<ChamberArgs> clr, stp, swr, swl;
        for (size_t i = 0; i < n; ++i) {
            agb_world* w = W[i];
            if (!world_emission_active(w)) continue;
            emit[i] = 1;
            ChamberArgs a = chamber_args(w);
            clr.push_back(a);
            if (w->c.source > 0.0f) stp.push_back(a);
            const GridDev& I = w->c.g[AGB_FIELD_IRRADIANCE];
            const int axis = w->c.light_axis;
            const int64_t len = axis == 0 ? I.nx : (axis == 1 ? I.ny : I.nz);
            const int64_t lines = I.count / len;
            if (axis == 0) {
                a.nblk = sweep_rows_blocks(lines);
                swr.push_back(a);
            } else {
                a.nblk = (int32_t)((lines + 127) / 128);
                swl.push_back(a);
            }
        }
        P.stage(1, BStage::ClearStamps, clr);
        P.stage(1, BStage::Stamp, stp);
        P.stage(1, BStage::Occlusion, stp);
        P.stage(1, BStage::SweepRows, swr);
        P.stage(1, BStage::SweepLines, swl);
    }
    P.record(1, 1);
    // Motion samples CO2 and N2 as they stand before this tick's slow fields.
    std::vector<Ctx> pre(n);
    for (size_t i = 0; i < n; ++i) {
        world_refresh(W[i]);
        pre[i] = W[i]->c;
    }
    // Branch 2: slow fields.
    for (int f : {AGB_FIELD_CO2, AGB_FIELD_N2}) {
        int32_t maxs = 0;
        for (const agb_world* w : W)
            if (w->c.g[f].enabled) maxs = std::max(maxs, f == AGB_FIELD_CO2 ? w->tp.c_substeps : w->tp.n_substeps);
        for (int32_t k = 0; k < maxs; ++k) {
            std::vector<agb_world*> act;
            for (agb_world* w : W)
                if (w->c.g[f].enabled && k < (f == AGB_FIELD_CO2 ? w->tp.c_substeps : w->tp.n_substeps))
                    act.push_back(w);
            plan_ftcs(P, 2, act, f);
        }
    }
    P.record(2, 2);
    // Main branch: the hash.
    {
        std::vector<ChamberArgs> hc, kh;
        int32_t maxp = 0;
        for (agb_world* w : W) {
            ChamberArgs a = chamber_args(w);
            kh.push_back(a);
            a.nblk = hash_clear_blocks(a.passes, a.max_tiles, a.radix_bits);
            hc.push_back(a);
            maxp = std::max(maxp, a.passes);
        }
        P.stage(0, BStage::HashClear, hc);
        P.stage(0, BStage::KeyHist, kh);
        for (int32_t p = 0; p < maxp; ++p) {
            std::vector<ChamberArgs> r4, r49, r8;
            for (size_t i = 0; i < n; ++i) {
                if (p >= kh[i].passes) continue;
                ChamberArgs a = kh[i];
                int32_t passes = 0, tiles = 0, rb = 8;
                bool per4 = true;
                hash_sort_shape(W[i]->c.h, W[i]->c.capacity, passes, tiles, per4, rb);
                a.nblk = tiles;
                (!per4 ? r8 : (rb == 9 ? r49 : r4)).push_back(a);
            }
            P.stage(0, BStage::Radix4, r4, p);
            P.stage(0, BStage::Radix4x9, r49, p);
            P.stage(0, BStage::Radix8, r8, p);
        }
        P.stage(0, BStage::Ranges, kh);
    }
    P.wait(0, 1);
    P.wait(0, 4);
    // Feeding, taxis and forces in one pass; then integration with the CO2 demand.
    {
        std::vector<ChamberArgs> cs, ig;
        for (size_t i = 0; i < n; ++i) {
            agb_world* w = W[i];
            ChamberArgs a = chamber_args(w);
            for (int f : {AGB_FIELD_CO2, AGB_FIELD_N2}) a.c.g[f] = pre[i].g[f];
            a.arg = (emit[i] ? 1 : 0) | (w->d.taxis_enabled ? 2 : 0);
            cs.push_back(a);
            a.g = w->c.g[AGB_FIELD_CO2];
            ig.push_back(a);
        }
        P.stage(0, BStage::CellStep, cs);
        P.wait(0, 2);
        P.stage(0, BStage::Integrate, ig);
    }
    // Lifecycle and, on compaction ticks, compaction.
    {
        std::vector<ChamberArgs> um, sc, dv, kp, sc1, ga, sw;
        for (agb_world* w : W) {
            ChamberArgs a = chamber_args(w);
            const bool compact = world_compaction_allowed(w);
            um.push_back(a);
            ChamberArgs d = a;
            d.arg = compact ? 1 : 0;
            dv.push_back(d);
            ChamberArgs q = a;
            q.nblk = scan_blocks(w->c.capacity);
            sc.push_back(q);
            if (compact) {
                kp.push_back(a);
                sc1.push_back(q);
                ChamberArgs one = a;
                one.nblk = 1;
                sw.push_back(one);
            }
        }
        P.stage(0, BStage::UptakeMark, um);
        P.stage(0, BStage::Scan, sc, 0);
        P.stage(0, BStage::Divide, dv);
        P.stage(0, BStage::Keep, kp);
        P.stage(0, BStage::Scan, sc1, 1);
        P.stage(0, BStage::ScatterSrc, kp);
        P.stage(0, BStage::Gather, kp);
        P.stage(0, BStage::Swap, sw);
    }
    for (agb_world* w : W) world_advance_clock(w, 1);
}

void run_plan(agb_batch* b, const StagedPlan& P, char* arena, cudaStream_t s) {
    cudaStream_t st[4] = {s, b->side[0], b->side[1], b->side[2]};
    for (const StagedOp& o : P.ops) {
        switch (o.kind) {
            case OpKind::Launch:
                launch_batched(o.st, reinterpret_cast<const ChamberArgs*>(arena + o.tab),
                               reinterpret_cast<const uint32_t*>(arena + o.map), o.blocks, o.arg, st[o.stream]);
                break;
            case OpKind::Ftcs:
                launch_ftcs_batch(reinterpret_cast<const FtcsChamber*>(arena + o.tab), o.nch, o.nx, o.ny, o.nz,
                                  o.plan, st[o.stream]);
                break;
            case OpKind::Record: cudaEventRecord(b->sev[o.event], st[o.stream]); break;
            case OpKind::Wait: cudaStreamWaitEvent(st[o.stream], b->sev[o.event], 0); break;
        }
    }
}

// Median ms per tick of `ticks` graph-replayed ticks. The warm-up runs two
// compaction periods of ticks first, so every (buffer parity, compaction
// phase) graph is captured before the timed ticks and no capture falls
// between their events.
float time_ticks(agb_world* w, int32_t ticks, cudaStream_t s) {
    const int32_t period = w->d.compaction_period > 0 ? w->d.compaction_period : 1;
    for (int32_t k = 0; k < 2 * period; ++k)
        if (agb_world_step_graph(w, 1, s) != AGB_OK) return -1.0f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<float> ms;
    for (int32_t k = 0; k < ticks; ++k) {
        cudaEventRecord(e0, s);
        if (agb_world_step_graph(w, 1, s) != AGB_OK) break;
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) break;
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        ms.push_back(t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms.empty()) return -1.0f;
    std::sort(ms.begin(), ms.end());
    return ms[ms.size() / 2];
}

struct ClassChoice {
    double hash_cell = 0.0;
    FtcsPlan plan[3] = {};
    bool tuned_plan[3] = {false, false, false};
    float tick_ms = 0.0f, pass_us = 0.0f;
};

// Chambers run concurrently, so each keeps one thread per cell in its
// neighbour walks (the other chambers fill the GPU); small ones still fuse
// feeding, taxis and forces into one pass. Measured on GB300 with 64 chambers
// of 2.6M cells: 3.85 ms/step at 1 lane fused, 4.33 at 2 lanes fused, 3.97
// at 1 lane as separate kernels.
static void batch_walk(agb_world* w) { w->walk_lanes = 1; }

// Time every candidate on probes built from one representative chamber.
agb_status tune_class(agb_batch* b, const agb_world_desc& rep, const agb_spawn& sp, const agb_batch_opts& o,
                      cudaStream_t s, ClassChoice* out) {
    std::vector<double> cands;
    for (int k = 0; k < o.n_hash_candidates && k < 8; ++k)
        if (o.hash_candidates[k] >= AGB_CELL_DIAMETER) cands.push_back(o.hash_candidates[k]);
    if (cands.empty())
        for (double f : {1.0, 1.5, 2.2, 3.0}) cands.push_back(f * AGB_CELL_DIAMETER);
    const int32_t ticks = o.probe_ticks > 0 ? o.probe_ticks : 4;
    float best = -1.0f;
    agb_world* keep = nullptr;
    for (double h : cands) {
        agb_world_desc d = rep;
        d.hash_cell_size = h;
        agb_world* w = nullptr;
        agb_status rc = agb_world_create(&d, &w);
        if (rc == AGB_UNSUPPORTED || rc == AGB_INVALID_ARGUMENT) continue;   // e.g. too many buckets
        if (rc != AGB_OK) return bfail(b, rc, "autotune: probe chamber");
        batch_walk(w);
        rc = agb_world_spawn(w, &sp, s);
        if (rc != AGB_OK) { agb_world_destroy(w); return bfail(b, rc, "autotune: probe spawn"); }
        const float t = time_ticks(w, ticks, s);
        if (t > 0.0f && (best < 0.0f || t < best)) {
            best = t;
            out->hash_cell = h;
            if (keep) agb_world_destroy(keep);
            keep = w;
        } else {
            agb_world_destroy(w);
        }
    }
    if (!keep) return bfail(b, AGB_CUDA_ERROR, "autotune: no hash cell candidate ran");
    out->tick_ms = best;
    // Stencil tilings on the kept probe's own grids (its field contents are
    // expendable).
    for (int f = 0; f < 3; ++f) {
        const agb_grid_desc& g = rep.grid[f];
        if (g.nx <= 0 || g.nz <= 1 || !keep->tmap_ok[f]) continue;
        float bp = -1.0f;
        const int32_t opts[5][2] = {{16, 1}, {16, 2}, {32, 1}, {32, 2}, {32, 4}};
        for (const auto& lr : opts) {
            if (lr[0] == 32 && g.nx < 128) continue;
            const FtcsPlan p = ftcs_plan_with(g.nx, g.ny, g.nz, lr[0], lr[1], 0);
            if (!world_set_tiling(keep, f, p)) continue;
            const float t = world_time_passes(keep, f, 8, s);
            if (t > 0.0f && (bp < 0.0f || t < bp)) { bp = t; out->plan[f] = p; out->tuned_plan[f] = true; }
        }
        if (f == AGB_FIELD_TEMPERATURE && bp > 0.0f) out->pass_us = 1000.0f * bp;
    }
    agb_world_destroy(keep);
    return cudaGetLastError() == cudaSuccess ? AGB_OK : bfail(b, AGB_CUDA_ERROR, "autotune");
}

}  // namespace

extern "C" {

void agb_batch_opts_default(agb_batch_opts* o) {
    if (!o) return;
    *o = agb_batch_opts{};
    o->abi_version = AGB_ABI_VERSION;
    o->lanes = 0;
    o->autotune = 0;
    o->n_hash_candidates = 0;
    o->probe_ticks = 4;
    o->staged = 1;
}

void agb_batch_destroy(agb_batch* b) {
    if (!b) return;
    drop_graphs(b);
    for (agb_world* w : b->worlds) agb_world_destroy(w);
    for (cudaStream_t st : b->lane_streams) if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : b->lane_join) if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    for (cudaStream_t st : b->side) if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : b->sev) if (e) cudaEventDestroy(e);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
}

agb_status agb_batch_create(const agb_world_desc* descs, const agb_spawn* spawns, int32_t n,
                            const agb_batch_opts* opts, agb_batch** out) {
    if (!out) return AGB_INVALID_ARGUMENT;
    *out = nullptr;
    if (!descs || n <= 0 || n > AGB_BATCH_MAX_CHAMBERS) return AGB_INVALID_ARGUMENT;
    agb_batch_opts o;
    agb_batch_opts_default(&o);
    if (opts) {
        if (opts->abi_version != AGB_ABI_VERSION) return AGB_CONTRACT_VERSION_MISMATCH;
        o = *opts;
    }
    agb_batch* b = new (std::nothrow) agb_batch();
    if (!b) return AGB_OUT_OF_MEMORY;
    b->tuning.assign((size_t)n, agb_tuning{});
    std::vector<agb_world_desc> d(descs, descs + n);
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        agb_batch_destroy(b);
        return AGB_CUDA_ERROR;
    }
    b->own_stream = s;

    // Size classes: temperature grid edge x decade of the spawned cell count.
    std::map<std::pair<int32_t, int32_t>, std::vector<int32_t>> classes;
    for (int32_t i = 0; i < n; ++i) {
        const int32_t cells = spawns ? spawns[i].count : 0;
        const int32_t dec = cells > 0 ? (int32_t)std::floor(std::log10((double)cells)) : -1;
        classes[{d[i].grid[AGB_FIELD_TEMPERATURE].nx, dec}].push_back(i);
    }
    std::vector<ClassChoice> choice((size_t)n);
    int32_t cls = 0;
    for (auto& kv : classes) {
        std::vector<int32_t>& mem = kv.second;
        std::sort(mem.begin(), mem.end(), [&](int32_t a, int32_t c) {
            return (spawns ? spawns[a].count : 0) < (spawns ? spawns[c].count : 0);
        });
        ClassChoice cc;
        if (o.autotune) {
            const int32_t r = mem[mem.size() / 2];
            agb_spawn sp{};
            if (spawns) sp = spawns[r];
            const agb_status rc = tune_class(b, d[r], sp, o, s, &cc);
            if (rc != AGB_OK) { agb_batch_destroy(b); return rc; }
        }
        for (int32_t i : mem) {
            choice[(size_t)i] = cc;
            b->tuning[(size_t)i].size_class = cls;
        }
        ++cls;
    }

    // The chambers, built with the tuned hash cells and tilings.
    b->worlds.assign((size_t)n, nullptr);
    for (int32_t i = 0; i < n; ++i) {
        agb_world_desc di = d[(size_t)i];
        if (choice[(size_t)i].hash_cell > 0.0) di.hash_cell_size = choice[(size_t)i].hash_cell;
        agb_status rc = agb_world_create(&di, &b->worlds[(size_t)i]);
        if (rc != AGB_OK) { agb_batch_destroy(b); return rc; }
        agb_world* w = b->worlds[(size_t)i];
        batch_walk(w);
        agb_tuning& t = b->tuning[(size_t)i];
        t.hash_cell_size = di.hash_cell_size > 0.0 ? di.hash_cell_size : AGB_HASH_CELL_FACTOR * AGB_CELL_DIAMETER;
        t.probe_tick_ms = choice[(size_t)i].tick_ms;
        t.probe_pass_us = choice[(size_t)i].pass_us;
        for (int f = 0; f < 3; ++f) {
            if (choice[(size_t)i].tuned_plan[f]) world_set_tiling(w, f, choice[(size_t)i].plan[f]);
            if (w->tmap_ok[f]) {
                t.ftcs_lx[f] = w->tplan[f].lx; t.ftcs_rpt[f] = w->tplan[f].rpt; t.ftcs_zc[f] = w->tplan[f].zc;
            }
        }
        if (spawns && spawns[i].count > 0) {
            rc = agb_world_spawn(w, &spawns[i], s);
            if (rc != AGB_OK) { agb_batch_destroy(b); return rc; }
        }
    }

    // Lanes: heaviest chamber first onto the least-loaded lane.
    b->lanes = o.lanes > 0 ? o.lanes : 16;
    if (b->lanes > n) b->lanes = n;
    std::vector<std::pair<double, int32_t>> load;
    for (int32_t i = 0; i < n; ++i) load.push_back({tick_bytes(d[(size_t)i], spawns ? spawns[i].count : 0), i});
    std::sort(load.begin(), load.end(), [](const auto& a, const auto& c) {
        return a.first > c.first || (a.first == c.first && a.second < c.second);
    });
    std::vector<double> lane_load((size_t)b->lanes, 0.0);
    for (const auto& li : load) {
        const int32_t l = (int32_t)(std::min_element(lane_load.begin(), lane_load.end()) - lane_load.begin());
        lane_load[(size_t)l] += li.first;
        b->tuning[(size_t)li.second].lane = l;
    }
    for (int32_t l = 0; l < b->lanes; ++l)
        for (int32_t i = 0; i < n; ++i)
            if (b->tuning[(size_t)i].lane == l) b->order.push_back(i);
    b->lane_streams.assign((size_t)b->lanes, nullptr);
    b->lane_join.assign((size_t)b->lanes, nullptr);
    bool ok = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int32_t l = 0; l < b->lanes && ok; ++l)
        ok = cudaStreamCreateWithFlags(&b->lane_streams[(size_t)l], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->lane_join[(size_t)l], cudaEventDisableTiming) == cudaSuccess;
    for (cudaStream_t& st : b->side)
        ok = ok && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t& e : b->sev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(s) == cudaSuccess;
    if (!ok) { agb_batch_destroy(b); return AGB_CUDA_ERROR; }
    // Staged ticks run every chamber's walks fused, one lane per cell.
    if (o.staged) {
        for (agb_world* w : b->worlds) w->fuse_cells = true;
        b->staged = staged_ok(b);
        if (!b->staged)
            for (agb_world* w : b->worlds) w->fuse_cells = (int64_t)w->c.capacity <= (int64_t)w->sm_count * 512;
    }
    *out = b;
    return AGB_OK;
}

const char* agb_batch_last_error(const agb_batch* b) { return b ? b->err.c_str() : ""; }

agb_status agb_batch_size(agb_batch* b, int32_t* n) {
    if (!b || !n) return AGB_INVALID_ARGUMENT;
    *n = (int32_t)b->worlds.size();
    return AGB_OK;
}

agb_status agb_batch_world(agb_batch* b, int32_t i, agb_world** w) {
    if (!b || !w || i < 0 || i >= (int32_t)b->worlds.size()) return AGB_INVALID_ARGUMENT;
    *w = b->worlds[(size_t)i];
    return AGB_OK;
}

agb_status agb_batch_tuning(agb_batch* b, int32_t i, agb_tuning* out) {
    if (!b || !out || i < 0 || i >= (int32_t)b->worlds.size()) return AGB_INVALID_ARGUMENT;
    *out = b->tuning[(size_t)i];
    return AGB_OK;
}

agb_status agb_batch_step(agb_batch* b, int32_t ticks, agb_stream stream) {
    if (!b || ticks <= 0) return AGB_INVALID_ARGUMENT;
    cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : b->own_stream;
    const std::vector<uint64_t> key = batch_key(b, ticks);
    for (const BatchGraph& g : b->graphs) {
        if (g.key != key) continue;
        const cudaError_t e = cudaGraphLaunch(g.exec, s);
        if (e != cudaSuccess) return bfail(b, AGB_CUDA_ERROR, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
        b->graph_kernels_total += g.kernels;
        for (size_t i = 0; i < b->worlds.size(); ++i) {
            world_set_parity(b->worlds[i], g.parity_after[i]);
            world_advance_clock(b->worlds[i], ticks);
        }
        return AGB_OK;
    }
    const bool staged = b->staged && staged_ok(b);
    StagedPlan plan;
    char* arena = nullptr;
    if (staged) {
        // Plan every tick (advancing the chambers' host state), then put the
        // tables in device memory before capturing the launches that read them.
        for (int32_t t = 0; t < ticks; ++t) plan_tick(b, plan);
        cudaError_t e = cudaMalloc(&arena, plan.bytes.size() > 0 ? plan.bytes.size() : 128);
        if (e == cudaSuccess && !plan.bytes.empty())
            e = cudaMemcpy(arena, plan.bytes.data(), plan.bytes.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (arena) cudaFree(arena);
            return bfail(b, AGB_CUDA_ERROR, std::string("staged tables: ") + cudaGetErrorString(e));
        }
    }
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        if (arena) cudaFree(arena);
        return bfail(b, AGB_CUDA_ERROR, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
    }
    if (staged) {
        run_plan(b, plan, arena, s);
    } else {
        // Fork every lane off s, run each lane's chambers one after the other
        // (each tick forks onto the chamber's own side streams), join.
        cudaEventRecord(b->fork, s);
        for (cudaStream_t ls : b->lane_streams) cudaStreamWaitEvent(ls, b->fork, 0);
        for (int32_t i : b->order) {
            agb_world* w = b->worlds[(size_t)i];
            cudaStream_t ls = b->lane_streams[(size_t)b->tuning[(size_t)i].lane];
            for (int32_t t = 0; t < ticks; ++t) world_tick(w, ls);
        }
        for (int32_t l = 0; l < b->lanes; ++l) {
            cudaEventRecord(b->lane_join[(size_t)l], b->lane_streams[(size_t)l]);
            cudaStreamWaitEvent(s, b->lane_join[(size_t)l], 0);
        }
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess) {
        if (arena) cudaFree(arena);
        return bfail(b, AGB_CUDA_ERROR, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    }
    BatchGraph bg{key, nullptr, {}, 0, arena};
    {
        size_t nn = 0;
        cudaGraphGetNodes(graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) cudaGraphGetNodes(graph, nodes.data(), &nn);
        for (auto nd : nodes) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++bg.kernels;
        }
    }
    e = cudaGraphInstantiate(&bg.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        if (arena) cudaFree(arena);
        return bfail(b, AGB_CUDA_ERROR, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    // Capture advanced each chamber's host-side state; the graph has not run yet.
    for (agb_world* w : b->worlds) bg.parity_after.push_back(world_parity(w));
    e = cudaGraphLaunch(bg.exec, s);
    b->graphs.push_back(std::move(bg));
    if (e != cudaSuccess) return bfail(b, AGB_CUDA_ERROR, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
    b->graph_kernels_total += b->graphs.back().kernels;
    return AGB_OK;
}

agb_status agb_batch_staged(agb_batch* b, int32_t* staged) {
    if (!b || !staged) return AGB_INVALID_ARGUMENT;
    *staged = (b->staged && staged_ok(b)) ? 1 : 0;
    return AGB_OK;
}

agb_status agb_batch_graph_kernels(agb_batch* b, int64_t* kernels) {
    if (!b || !kernels) return AGB_INVALID_ARGUMENT;
    *kernels = b->graph_kernels_total;
    return AGB_OK;
}

agb_status agb_batch_stats(agb_batch* b, agb_stats* out) {
    if (!b || !out) return AGB_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(b->own_stream) != cudaSuccess) return AGB_CUDA_ERROR;
    for (size_t i = 0; i < b->worlds.size(); ++i) {
        const agb_status rc = agb_world_stats(b->worlds[i], &out[i], nullptr);
        if (rc != AGB_OK) return rc;
    }
    return AGB_OK;
}

}  // extern "C"
