// world.cuh -- per-world constants (Ctx, passed by value to kernels) and the
// host-side world object behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "dev.cuh"

namespace agb {

// Everything a kernel needs that does not change during a tick.
struct Ctx {
    GridDev g[AGB_FIELD_COUNT];
    HashDev h;
    double chamber_w, chamber_h, chamber_d;
    int32_t capacity;
    uint64_t seed;
    int32_t boundary_x, boundary_y, gravity_axis;
    int32_t thermal_noise, contact_enabled, adhesion_enabled, occlusion_exact;
    int32_t store_disposition, division_predicate;
    double division_energy, co2_quota;
    int32_t trap_slot;
    double trap_x, trap_y;
    // Wall limits of apply_boundary_axis (src/sim/integrator.cuh:233-254) per axis.
    double lo[3], hi[3], half[3];
    unsigned long long lo_key[3], hi_key[3];
    // Light (src/sim/emission.cu:140-165)
    float lx, ly, lz;          // unit light direction as float
    double ldx, ldy, ldz;      // ... and as double (reference normalize)
    int32_t light_axis, light_sign;
    int32_t light_axis_exact;  // light exactly along light_axis (other components 0), else -1
    float source, ambient_irr;
    double source_d;           // (double)source
    // One byte per irradiance line of the sweep: 1 = a cell stamped a voxel of
    // it this tick, 2 = stamped last tick only (recompute once to clear the old
    // shadow), 0 = no stamp in either, so its values are already the
    // unshadowed ones and the sweep leaves it alone. Null: sweep every line.
    uint8_t* irr_marks;
    // One bit per irradiance voxel: set where this tick's stamps deposited
    // (mirrors deposit != 0), so the sweep tests bits instead of reading the
    // 8-byte deposit of every voxel.
    uint32_t* irr_stamp_bits;
    int32_t* t_vox;          // per slot: its temperature voxel, written by a tick's first thermal substep and read
                             // by the later substeps and flushes (cells do not move in between); null: recompute
    double face_area;
    long long stamp_alive, stamp_dead;   // fixed-point occlusion stamps
    // Occlusion factors of the commonest stamped voxels (one, two or three
    // live cells, or one dead cell), computed on the host with the same FP64
    // operations as the device, which looks these deposits up instead of
    // dividing.
    unsigned long long occl_dep[4];
    double occl_fac[4];
    // Exact float thresholds equivalent to the reference's FP64 compares.
    float setpoint_up;          // smallest float >= CELL_TEMP_SETPOINT
    float setpoint_hi, setpoint_lo;
    float lethal_f;             // t_local > CELL_LETHAL_TEMP  <=>  t_local > lethal_f
    uint64_t stick_bits;        // uniform53 < stick_bits  <=>  uniform01d < WALL_STICKINESS
};

// Per-tick scalars derived from the clock.
struct TickParams {
    double dt;                  // DT_PHYSICS * physics_rate
    double dt_inv;              // 1 / dt, rounded once (div_known)
    float dtf;
    float k_contact;            // CONTACT_STIFFNESS / physics_rate
    double k_contact64;
    float k_trap;
    double dt_bio;
    float dt_bio_f;             // (float)dt_bio
    // thermal
    int32_t t_substeps;
    double t_dt_sub;
    float t_coeff;
    float t_cap_relax;          // capacity * (1 - exp(-G dt_sub / C)) as float
    float t_relax;              // (1 - exp(-G dt_sub / C)) as float
    double t_cap;
    // taxis
    double taxis_alpha;         // 1 - exp(-dt / TAXIS_MEMORY_TIME) (taxis.cuh:38-41)
    double max_emit_power;      // [W]
    // slow fields
    int32_t c_substeps, n_substeps;
    float c_coeff, n_coeff;
};

}  // namespace agb
