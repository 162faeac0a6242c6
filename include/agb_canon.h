/*
 * include/agb_canon.h -- the physical constants the per-tick physics reads.
 *
 * These are DATA, not code: the values the simulator's canon generator emits
 * (src/core/canon_generated.h:12-146) and the fixed-point scales of the fields
 * contract (contracts/fields_v1.h:47-78), repeated value for value because
 * bit-level parity with the reference needs the identical doubles. Plain C so
 * the CUDA engine, its C++ host code and the C oracle all read one table.
 */
#ifndef AGB_CANON_H
#define AGB_CANON_H

/* Universal constants (canon_generated.h:12-19). */
#define AGB_C_LIGHT 299792458.0
#define AGB_PETROVA_FLASH_POWER 3000000.0          /* canon_generated.h:33, spin-drive discharge [W] */
/* Fixed-point scales of the flash audit (src/sim/flash.cu:24-27). */
#define AGB_FLASH_IMPULSE_SCALE 1.0e15
#define AGB_FLASH_ENERGY_SCALE 1.0e6
#define AGB_K_BOLTZ 1.3806490000000001e-23
#define AGB_G_ACCEL 9.8066499999999994

/* Cell (canon_generated.h:22-28, 94-101). */
#define AGB_CELL_DIAMETER 1.0000000000000001e-05
#define AGB_CELL_RADIUS 5.0000000000000004e-06
#define AGB_CELL_MASS_DRY 2.0999999999999999e-14
#define AGB_CELL_TEMP_SETPOINT 369.565
#define AGB_CELL_ENERGY_MAX 1500000.0
#define AGB_CELL_ALBEDO_DEAD 0.84999999999999998
#define AGB_CELL_LETHAL_TEMP 573.14999999999998
#define AGB_CELL_VOLUME 5.2359877559829892e-16
#define AGB_CELL_CROSS_SECTION 7.8539816339744834e-11
#define AGB_CELL_SURFACE_AREA 3.1415926535897934e-10

/* Biology (canon_generated.h:36-42, 122-123). */
#define AGB_CO2_MASS_PER_DIVISION 2.0999999999999999e-14
#define AGB_CO2_DIFFUSIVITY_WATER 1.92e-09
#define AGB_LIFE_DIVISION_ENERGY_COST 0.0
#define AGB_LIFE_CO2_HALF_SATURATION 0.001
#define AGB_LIFE_CO2_UPTAKE_MAX 3.0381944444444441e-20

/* Water and heat (canon_generated.h:53-63, 108-114). */
#define AGB_WATER_DENSITY 998.20000000000005
#define AGB_WATER_CONDUCTIVITY 0.59799999999999998
#define AGB_WATER_SPECIFIC_HEAT 4182.0
#define AGB_WATER_BOILING_POINT 373.14999999999998
#define AGB_VF_A 2.4139999999999999e-05
#define AGB_VF_B 570.58000000000004
#define AGB_VF_C 140.0
#define AGB_AIR_CONVECTION_H 10.0
#define AGB_AMBIENT_TEMP_DEFAULT 293.14999999999998
#define AGB_WATER_THERMAL_DIFFUSIVITY 1.4325163582348751e-07
#define AGB_CONDUCTION_COEFF 3.7573448136933928e-05

/* Mechanics (canon_generated.h:64-69). */
#define AGB_CONTACT_STIFFNESS 1.1802e-05
#define AGB_WALL_STICKINESS 0.14999999999999999
#define AGB_WALL_STUCK_DRAG_MULT 20.0
#define AGB_WALL_RELEASE_FORCE 5.0000000000000002e-11
#define AGB_HASH_CELL_FACTOR 2.2000000000000002
#define AGB_DT_PHYSICS 0.001

/* Clocks (canon_generated.h:70-73). */
#define AGB_CLOCK_PHYSICS_MIN 0.10000000000000001
#define AGB_CLOCK_PHYSICS_MAX 100.0
#define AGB_CLOCK_BIOLOGY_MIN 1.0
#define AGB_CLOCK_BIOLOGY_MAX 1000000.0
/* Clock presets (canon_generated.h:74-81). */
#define AGB_CLOCK_REALTIME_PHYSICS 1.0
#define AGB_CLOCK_REALTIME_BIOLOGY 1.0
#define AGB_CLOCK_MOTION_PHYSICS 10.0
#define AGB_CLOCK_MOTION_BIOLOGY 1.0
#define AGB_CLOCK_METABOLIC_PHYSICS 1.0
#define AGB_CLOCK_METABOLIC_BIOLOGY 10000.0
#define AGB_CLOCK_GENERATIONAL_PHYSICS 0.5
#define AGB_CLOCK_GENERATIONAL_BIOLOGY 1000000.0

/* Chamber and grids (canon_generated.h:87-89, 135-141). */
#define AGB_CHAMBER_W 0.0040000000000000001
#define AGB_CHAMBER_H 0.0040000000000000001
#define AGB_CHAMBER_D 6.0000000000000002e-05
#define AGB_FIELD_N_TEMP 512
#define AGB_FIELD_N_CO2 256
#define AGB_FIELD_N_N2 128
#define AGB_FIELD_N_IRRAD 512
#define AGB_MAX_CELLS 2000000
#define AGB_DEFAULT_CELLS 25000
#define AGB_DEFAULT_TAUMOEBA 256
#define AGB_MAX_TAUMOEBA 65536
/* Run-and-tumble taxis (src/core/canon_generated.h:31,82-86,120). */
#define AGB_PETROVA_MAX_POWER 0.050000000000000003
#define AGB_TAXIS_MEMORY_TIME 0.10000000000000001
#define AGB_TAXIS_DARK_THRESHOLD 0.001
#define AGB_TAXIS_SEEK_FEED_BELOW 0.94999999999999996
#define AGB_TAXIS_SEEK_BREED_ABOVE 0.97999999999999998
#define AGB_TAXIS_TUMBLE_ANGLE_MEAN 1.1868238913561442
#define AGB_TAXIS_RUN_MAX 0.40000000000000002          /* predator store capacity of a world that sets none */
#define AGB_N2_DIFFUSIVITY 2.0e-9            /* src/sim/step.cu:38 literal */

/* Fixed-point scales (contracts/fields_v1.h:47-70; stats field scale src/sim/stats.cu:19). */
#define AGB_DEPOSIT_SCALE_TEMPERATURE 1.0e9
#define AGB_DEPOSIT_SCALE_CO2 1.0e15
#define AGB_DEPOSIT_SCALE_N2 1.0e15
#define AGB_DEPOSIT_SCALE_STATS 1.0e6
#define AGB_DEPOSIT_SCALE_IRRADIANCE 1.0e18
#define AGB_STATS_SCALE_FIELD 1.0e9
#define AGB_IRRADIANCE_NOMINAL_DIFFUSIVITY 1.0e-9

/* Mathematical constants (src/core/units.h:32-33). */
#define AGB_PI 3.14159265358979323846
#define AGB_TWO_PI 6.28318530717958647693

/* Cell flags and death causes (contracts/cell_store_v1.h:20-33). */
#define AGB_FLAG_OCCUPIED 0x1u
#define AGB_FLAG_ALIVE 0x2u
#define AGB_FLAG_AWAKE 0x4u
#define AGB_FLAG_STUCK 0x8u
#define AGB_FLAG_DIVIDING 0x10u
#define AGB_FLAG_FLASHING 0x20u
#define AGB_DEATH_NONE 0
#define AGB_DEATH_STARVED 1
#define AGB_DEATH_PREDATED 2
#define AGB_DEATH_OVERHEATED 3
#define AGB_DEATH_CULLED 4

#endif /* AGB_CANON_H */
