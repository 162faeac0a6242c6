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
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
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
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
    b->graphs.clear();
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
}

void agb_batch_destroy(agb_batch* b) {
    if (!b) return;
    drop_graphs(b);
    for (agb_world* w : b->worlds) agb_world_destroy(w);
    for (cudaStream_t st : b->lane_streams) if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : b->lane_join) if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
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
    ok = ok && cudaStreamSynchronize(s) == cudaSuccess;
    if (!ok) { agb_batch_destroy(b); return AGB_CUDA_ERROR; }
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
    // Capture: fork every lane off s, run each lane's chambers one after the
    // other (each tick forks onto the chamber's own side streams), join.
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bfail(b, AGB_CUDA_ERROR, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
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
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess) return bfail(b, AGB_CUDA_ERROR, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    BatchGraph bg{key, nullptr, {}, 0};
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
    if (e != cudaSuccess) return bfail(b, AGB_CUDA_ERROR, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    // Capture advanced each chamber's host-side state; the graph has not run yet.
    for (agb_world* w : b->worlds) bg.parity_after.push_back(world_parity(w));
    e = cudaGraphLaunch(bg.exec, s);
    b->graphs.push_back(std::move(bg));
    if (e != cudaSuccess) return bfail(b, AGB_CUDA_ERROR, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
    b->graph_kernels_total += b->graphs.back().kernels;
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
