/*
 * nwgb.h — C ABI of the GB300 nematic-worm step engine (libnwgb.so).
 *
 * One simulation step of self-propelled bead-spring filaments ("worms"),
 * optionally coupled to a stochastic-rotation-dynamics (SRD) solvent:
 *
 *   integrate(r, v | f, f_old) -> [reverse] -> Langevin -> bonded (bend,
 *   tangents, [bond, drive]) -> cell hash -> stable sort -> cell bounds ->
 *   pair forces -> [every srd_gap steps: SRD stream + rotate-collide]
 *
 * This is the order of ParticleSystem::update in the reference
 * (simulation/particleSystem.cpp:249-339) and of its SRD sub-step
 * (simulation/particleSystem.cpp:341-413).
 *
 * Two pair-force models share one kernel skeleton:
 *   NW_MODEL_WCA_WORMS  WCA Lennard-Jones between beads, harmonic bonds to
 *                       chain neighbours, k(1-cos) bending, tangent drive
 *                       F_act * unit(r_{i+1} - r_i), Langevin noise
 *                       sqrt(2 gamma kT / dt).  Force laws of the archived
 *                       engine (archived/vs_solution/fluid_substrate/
 *                       NWDeviceFunctions.h:65-76, NWWormsKernel_InternalForce.h:37-59
 *                       and 196-214, NWWormsKernel_BondBending.h:31-80,
 *                       NWWormsKernel_DriveForce.h:21-34, NWWormsParameters.h:135-156).
 *   NW_MODEL_REF_DEM    The modern engine's collideFilaments semantics:
 *                       DEM spring/dashpot/shear contact, Hookean bond found
 *                       through the cell list, extensile drive between
 *                       anti-aligned beads, noise sqrt(2 gamma kT)
 *                       (simulation/particles_kernel_impl.cuh:426-556, 694-744).
 *
 * Every entry point returns an nw_status; nothing in the library calls exit().
 * State arrays are float4 (x, y, z, w) per particle, the reference layout
 * (simulation/particleSystem.cpp:197-211): position.w = radius,
 * velocity.w = mass.
 */
#ifndef NWGB_H
#define NWGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NW_ABI_VERSION 2u

typedef int nw_status;
enum {
    NW_OK = 0,
    NW_ERR_CUDA = 1,          /* a CUDA runtime call failed */
    NW_ERR_INVALID = 2,       /* bad argument or configuration */
    NW_ERR_CELL_OVERFLOW = 3, /* a cell or neighbour list held more particles than its capacity */
    NW_ERR_NONFINITE = 4,     /* a non-finite position or force was produced */
    NW_ERR_TIMEOUT = 5,       /* a bounded device wait gave up */
    NW_ERR_NOMEM = 6,         /* device or host allocation failed */
    NW_ERR_UNSUPPORTED = 7,   /* feature not available in this configuration */
    NW_ERR_NO_DEVICE = 8,     /* no CUDA device visible */
    NW_ERR_IO = 9             /* a file could not be opened or written */
};

/* Device error word bits (read with nw_error_word). */
enum {
    NW_EFLAG_NONFINITE = 1u << 0,
    NW_EFLAG_CELL_OVERFLOW = 1u << 1,
    NW_EFLAG_TIMEOUT = 1u << 2,
    NW_EFLAG_BAD_INDEX = 1u << 3,
    NW_EFLAG_NEIGHBOR_OVERFLOW = 1u << 4
};

typedef enum { NW_MODEL_WCA_WORMS = 0, NW_MODEL_REF_DEM = 1 } nw_model;

/* Same numeric values as the reference's BoundaryType
 * (simulation/particles_kernel.cuh:18-23). */
typedef enum { NW_PERIODIC = 0, NW_WALL = 1, NW_WALL_NO_SLIP = 2 } nw_boundary;

/* Cell-hash wrap rule.  NW_HASH_MASK is the reference's power-of-two mask
 * (simulation/particles_kernel_impl.cuh:252-258); NW_HASH_MODULO wraps
 * periodic axes with a true modulo and clamps wall axes. */
typedef enum { NW_HASH_MODULO = 0, NW_HASH_MASK = 1 } nw_hash_mode;

/* SRD cell thermostat.
 *  NONE      no velocity rescaling.
 *  REF_LAB   the reference's isokinetic rule: every particle of a cell is
 *            scaled in the lab frame so that the cell's total kinetic energy
 *            equals kT (simulation/particles_kernel_impl.cuh:605-637); it
 *            runs before the cell mean is taken.
 *  CELL_REL  relative velocities (v - u_cell) are rescaled after the
 *            rotation so that their kinetic energy is (n_cell - 1) kT
 *            (two rotated degrees of freedom per particle). */
typedef enum { NW_SRD_THERMO_NONE = 0, NW_SRD_THERMO_REF_LAB = 1, NW_SRD_THERMO_CELL_REL = 2 } nw_srd_thermostat;

typedef struct NwConfig {
    uint32_t abi_version;      /* must be NW_ABI_VERSION */
    int32_t  model;            /* nw_model */
    int32_t  dim;              /* 2: noise and SRD shift have no z part, and WCA_WORMS
                                  systems compute in the xy plane (bead z and z velocity
                                  carried unchanged, forces with z = 0, as the archived
                                  two-component kernels); 3: full 3D */
    uint32_t num_filaments;
    uint32_t filament_size;    /* beads per filament, >= 1 */
    uint32_t grid[3];          /* bead cell grid */
    float    cell_size[3];
    float    origin[3];
    float    box[3];           /* grid * cell_size */
    int32_t  boundary[3];      /* nw_boundary per axis */
    int32_t  hash_mode;        /* nw_hash_mode */
    float    radius;           /* bead radius (position.w); DEM contact distance 2*radius */
    float    mass;             /* bead mass (velocity.w) */
    /* bonded terms */
    float    bond_k;           /* harmonic bond constant */
    float    bond_r0;          /* bond rest length */
    float    bend_k;           /* bending constant of U = k (1 - cos theta) */
    /* WCA_WORMS pair law */
    float    lj_epsilon;
    float    lj_sigma;
    float    lj_rcut;          /* cut-off; 2^(1/6) sigma gives WCA */
    int32_t  lj_exclude;       /* same-filament pairs with |i - j| <= lj_exclude are skipped */
    /* REF_DEM pair law */
    float    spring;
    float    damping;
    float    shear;
    float    attraction;       /* unused by the reference (commented out) */
    float    boundary_damping; /* velocity factor of a damped wall */
    /* activity */
    float    activity;         /* WCA: tangent drive F_act; REF: extensile amplitude */
    float    reverse_probability;
    /* Langevin thermostat */
    float    gamma;
    float    kT;
    int32_t  noise_dt_scaling; /* 1: sigma = sqrt(2 gamma kT / dt); 0: sqrt(2 gamma kT) */
    int32_t  langevin_with_srd;/* 0: Langevin only when the solvent is off (reference) */
    float    gravity[3];       /* stored for the API; the reference never applies it */
    /* SRD solvent */
    int32_t  srd_enabled;
    uint32_t num_solvent;
    uint32_t srd_grid[3];
    float    srd_cell_size[3];
    float    srd_alpha;        /* rotation angle, radians */
    uint32_t srd_gap;          /* collide every srd_gap steps; solvent streams gap*dt */
    float    srd_kT;
    float    solvent_mass;
    float    srd_shift_lo;     /* grid shift drawn in [lo, lo + 1) * srd_cell_size */
    int32_t  srd_rotate_beads; /* 1: beads are rotated with the solvent; 0: beads only enter the mean */
    int32_t  srd_thermostat;   /* nw_srd_thermostat */
    /* run control */
    uint64_t seed;
    float    dt;
    int32_t  strategy;         /* nw_strategy: how a step finds its neighbours */
    uint32_t cell_capacity;    /* beads a cell list holds (CELL_LISTS, VERLET): 8 or 16; 0 = by model */
    float    neighbor_skin;    /* VERLET: list radius = lj_rcut + skin; 0 = 0.3 lj_sigma */
    uint32_t neighbor_capacity;/* VERLET: neighbours a bead's list holds; 0 = 32 */
    uint32_t reserved[3];
} NwConfig;

/* Neighbour search of the bead step.
 *  SORTED      stable counting sort of the beads by cell, cell start/end and
 *              cell-ordered copies every step (the reference's scheme); five
 *              kernels per step, no occupancy limit.
 *  CELL_LISTS  capped per-cell bead lists; the pair pass of one step and the
 *              integrate/bonded pass of the next run as one kernel; the
 *              sorted order and cell bounds are produced only when read.
 *              A cell with more beads than cell_capacity is reported as
 *              NW_ERR_CELL_OVERFLOW.
 *  VERLET      (WCA_WORMS) CELL_LISTS on cells of at least lj_rcut + skin,
 *              from which each bead keeps the list of beads within that
 *              radius; steps reuse the lists while the summed maximum bead
 *              displacement since they were built stays below skin / 2, so
 *              every pair within lj_rcut is on them, and rebuild them in the
 *              pair pass otherwise.  Same forces as CELL_LISTS up to the
 *              order of the FP32 sums.
 *  AUTO        VERLET for WCA_WORMS, SORTED for REF_DEM (whose pair set is
 *              all beads of the neighbour cells, not a radius; its sorted
 *              pair pass on a single z layer runs cell-tiled in shared
 *              memory). */
typedef enum {
    NW_STRATEGY_AUTO = 0,
    NW_STRATEGY_SORTED = 1,
    NW_STRATEGY_CELL_LISTS = 2,
    NW_STRATEGY_VERLET = 3
} nw_strategy;

/* Array selectors for nw_get_array / nw_set_array / nw_device_array. */
typedef enum {
    NW_POSITION = 0,      /* float4[n_total]  (beads then solvent) */
    NW_VELOCITY = 1,      /* float4[n_total] */
    NW_TANGENT = 2,       /* float4[n_beads]  (WCA worms of more than three beads on the
                             cell-list / Verlet paths: computed from the current positions
                             when read, the step does not store them) */
    NW_FORCE = 3,         /* float4[n_beads] */
    NW_FORCE_OLD = 4,     /* float4[n_beads] */
    NW_HASH = 5,          /* uint[n_beads]   bead cell hash of the last step (unsorted order) */
    NW_SORTED_INDEX = 6,  /* uint[n_beads]   bead indices in stable cell order */
    NW_CELL_START = 7,    /* uint[n_cells]   0xffffffff for empty cells */
    NW_CELL_END = 8,      /* uint[n_cells]   valid where cell start is not empty */
    NW_SRD_SORTED_INDEX = 9, /* uint[n_total] indices of the last SRD collision, stable cell order */
    NW_SRD_CELL_START = 10,  /* uint[n_srd_cells] */
    NW_SRD_CELL_END = 11,    /* uint[n_srd_cells] */
    NW_SRD_CELL_MEAN = 12    /* float4[n_srd_cells] mass-weighted cell velocity of the last collision */
} nw_array;

typedef struct nw_system nw_system;

/* ---- configuration ---------------------------------------------------- */

/* Fill *cfg with the defaults of a model.  NW_MODEL_REF_DEM gives the
 * reference ParticleSystem constructor defaults
 * (simulation/particleSystem.cpp:39-111, 124-148) for the given grid;
 * NW_MODEL_WCA_WORMS gives the small 2D worm workload (400 x 10 beads in a
 * periodic 100 x 100 box, WCA eps = sigma = 1, bond k = 57, r0 = 0.8,
 * bend k = 10, F_act = 0.5, gamma = 2, kT = 0.1, dt = 0.005). */
nw_status nw_config_default(NwConfig* cfg, int model, uint32_t num_filaments,
                            uint32_t filament_size, uint32_t gx, uint32_t gy, uint32_t gz,
                            int srd);

/* Re-derive box/origin/cell fields after the caller changed grid or cell size
 * (origin = -box/2 as in simulation/particleSystem.cpp:76-79). */
nw_status nw_config_finalize(NwConfig* cfg);
/* Replaces: ParticleSystem::reset (simulation/particleSystem.cpp:583-678).
 * The reference's initial state for cfg into host arrays of (beads + solvent)
 * x 4 floats (pos, vel) and beads x 4 floats (tan): filaments along x on a
 * lattice of bond_r0 spacing, every other one (by draw) reversed, bead
 * velocities 0.1 U(-1, 1), solvent uniform in the box with velocities
 * 5 U(-1, 1), all drawn from the C library's rand() after srand(1) (the
 * reference never seeds it).  Host only; resets rand()'s state. */
nw_status nw_reference_reset(const NwConfig* cfg, float* pos, float* vel, float* tan);

/* Check a configuration without creating anything. */
nw_status nw_config_validate(const NwConfig* cfg);

/* ---- system lifetime ------------------------------------------------------ */

/* Replaces: ParticleSystem::ParticleSystem / _initialize
 * (simulation/particleSystem.cpp:39-111, 172-223).  Allocates every device
 * buffer once; nw_step never allocates. */
nw_status nw_create(const NwConfig* cfg, nw_system** out);
/* Replaces: ParticleSystem::~ParticleSystem / _finalize
 * (simulation/particleSystem.cpp:113-117, 225-246); frees everything. */
nw_status nw_destroy(nw_system* sys);

/* Replaces the ParticleSystem setters + setParameters upload
 * (simulation/particleSystem.h:53-121, particleSystem_cuda.cu:92-102).
 * Sizes (filaments, beads, solvent, grids) must not change. */
nw_status nw_set_config(nw_system* sys, const NwConfig* cfg);
nw_status nw_get_config(const nw_system* sys, NwConfig* cfg);

/* Counts. */
nw_status nw_get_counts(const nw_system* sys, uint32_t* n_beads, uint32_t* n_solvent,
                        uint32_t* n_cells, uint32_t* n_srd_cells);

/* ---- state transfer ------------------------------------------------------- */

/* Replaces: ParticleSystem::setArray (simulation/particleSystem.cpp:561-581).
 * Copies `count` elements (float4 or uint) from host memory, starting at
 * element `start`.  Synchronous with respect to the system's stream. */
nw_status nw_set_array(nw_system* sys, int array, const void* host, uint32_t start, uint32_t count);
/* Replaces: ParticleSystem::getArray (simulation/particleSystem.cpp:534-559). */
nw_status nw_get_array(nw_system* sys, int array, void* host, uint32_t start, uint32_t count);
/* nw_set_array / nw_get_array enqueued on the system's stream without waiting
 * (no counterpart in the reference, whose copies are synchronous): the host
 * buffer must stay untouched until nw_sync returns, and is best pinned, so
 * that the copies of a step (inputs, nw_step, results) run back to back on the
 * device with one synchronisation.  Arrays computed when read (sorted order,
 * cell bounds, reference hashes, tangents of lazy systems) are produced on the
 * stream as well. */
nw_status nw_set_array_async(nw_system* sys, int array, const void* host, uint32_t start, uint32_t count);
nw_status nw_get_array_async(nw_system* sys, int array, void* host, uint32_t start, uint32_t count);
/* Device pointer of an array (zero-copy access; valid until nw_destroy).  The
 * double-buffered state of the cell-list / Verlet paths moves between two
 * buffers with the step parity: ask again after stepping.  NW_POSITION marks
 * the neighbour lists for rebuilding (the caller may move beads through it). */
nw_status nw_device_array(nw_system* sys, int array, void** dptr);
/* Zero forces, old forces and the step counter (the reference never zeroes
 * them: simulation/particleSystem.cpp:202-203). */
nw_status nw_zero_forces(nw_system* sys);

/* ---- stepping ------------------------------------------------------------- */

/* Replaces: ParticleSystem::update (simulation/particleSystem.cpp:249-339),
 * nsteps times with step size dt (dt <= 0 uses cfg.dt).  Asynchronous on the
 * system's stream; runs from a cached CUDA graph when nsteps > 1. */
nw_status nw_step(nw_system* sys, int nsteps, float dt);
/* Capture, without running anything, the CUDA graph that nw_step(sys, nsteps,
 * dt) replays when called at update index first_step (only its SRD phase
 * matters), so that a later nw_step pays no capture.  No counterpart in the
 * reference; a no-op when graphs are off. */
nw_status nw_step_prepare(nw_system* sys, int nsteps, float dt, uint64_t first_step);
/* Wait for the stream, then report and clear the device error word. */
nw_status nw_sync(nw_system* sys);
nw_status nw_error_word(nw_system* sys, uint32_t* flags);
nw_status nw_get_step(const nw_system* sys, uint64_t* step);
nw_status nw_set_step(nw_system* sys, uint64_t step);
/* Use a caller stream (cudaStream_t passed as void*); NULL restores the
 * system's own stream. */
nw_status nw_set_stream(nw_system* sys, void* stream);
/* Enable or disable CUDA-graph replay for multi-step calls (default on). */
nw_status nw_set_graphs(nw_system* sys, int enabled);
/* Run only the SRD sub-step (for tests): shift given in world units. */
nw_status nw_srd_collide(nw_system* sys, float dt_srd, const float shift[3]);

/* ---- checkpoint / resume -------------------------------------------------- */

/* Bytes needed by nw_checkpoint_save. */
nw_status nw_checkpoint_size(const nw_system* sys, size_t* bytes);
/* Binary snapshot: config, step counter, positions, velocities, forces,
 * old forces, tangents.  Resuming from it is bit-exact. */
nw_status nw_checkpoint_save(nw_system* sys, void* host_buf, size_t bytes);
nw_status nw_checkpoint_load(nw_system* sys, const void* host_buf, size_t bytes);

/* ---- misc ----------------------------------------------------------------- */

const char* nw_status_string(nw_status s);
uint32_t nw_abi_version(void);
/* sizeof(NwConfig) as compiled into the library (binding layout check). */
size_t nw_config_size(void);
/* Number of kernels the last nw_step call launched (graph replays count the
 * kernels inside the graph). */
nw_status nw_last_launch_count(const nw_system* sys, uint64_t* launches);

/* Per-kernel device time of `nsteps` steps (direct launches, a CUDA event
 * before every kernel), aggregated by kernel name.  Advances the system like
 * nw_step.  Replaces the reference's host-clock phase counters
 * (archived/vs_solution/fluid_substrate/NWWorms.h:637-654). */
typedef struct NwKernelTime {
    char name[32];
    double total_ms;
    uint64_t launches;
} NwKernelTime;
nw_status nw_profile_steps(nw_system* sys, int nsteps, float dt, NwKernelTime* out, int max_entries, int* n_entries);

/* ---- trajectory output ---------------------------------------------------- */

/* Frames in the reference's text format (ParticleSystem::writeOutputs,
 * simulation/particleSystem.cpp:481-532, read by analysis/afa/io.py:4-25):
 * a line with the particle count, a line with the parameters as a JSON
 * object, then one line per particle, "A x y z vx vy vz" for beads and
 * "B x y z vx vy vz" for solvent (floats as C++ streams print them, 6
 * significant digits).  Unlike the reference, the frame leaves the step
 * loop at once: nw_writer_frame enqueues a device-to-device snapshot of the
 * state on the system's stream, the writer copies it to pinned host memory
 * on its own stream, and a writer thread formats and appends it to the
 * file.  Two frames can be in flight; a third call waits for the oldest.
 * Close every writer before destroying its system. */
typedef struct nw_writer nw_writer;
nw_status nw_writer_open(nw_system* sys, const char* path, int append, nw_writer** out);
/* Snapshot of the current state, written as iteration `iteration` with
 * time step dt (the JSON's "time" is iteration * dt). */
nw_status nw_writer_frame(nw_writer* w, int iteration, float dt);
/* Wait until every enqueued frame is in the file; reports a write failure. */
nw_status nw_writer_flush(nw_writer* w);
nw_status nw_writer_close(nw_writer* w);

/* ---- topological defects -------------------------------------------------- */

/* +1/2 and -1/2 defects of the nematic director field of a 2D system, the
 * reference's analysis (analysis/make_director_field.py:10-47 then
 * analysis/find_defects.py:43-207) on the current bead positions:
 *  - bead tangents r_{i+1} - r_{i-1}, one-sided at filament ends; the first
 *    and the last bead of the system get none (analysis/afa/utils.py:35-49
 *    centres its windows on beads 1 .. n-2); raw differences unless
 *    NW_DEFECT_MIN_IMAGE asks for the minimum image;
 *  - a grid of cells of edge cell_size from the beads' lowest x and y,
 *    ceil((max - min + 1e-4) / cell_size) cells per axis;
 *  - a cell's director angle is the nematic tensor's, taken in
 *    [-pi/4, 3pi/4) (-pi/2 for a vertical director, 0 for an empty cell),
 *    the representative the reference's eigen-solver gives;
 *  - around every interior cell the director's rotation along the ring of its
 *    8 neighbours, each step taken into (-pi/2, pi/2); a total beyond
 *    pi - pi/16 in magnitude marks a defect cell of charge sign / 2;
 *  - marked cells of one sign that touch (8-neighbourhood, no periodic wrap)
 *    form one defect at (mean cell index) * cell_size + min + cell_size / 2.
 * Positive defects first, each sign in order of its first cell (x-major).
 * Binning (fixed-point sums: independent of thread order) and the circuits
 * run on the device, the clustering of the marked cells on the host.
 * Synchronous.  *n_out is the number of defects; at most max_out are written. */
#define NW_DEFECT_MIN_IMAGE 1u
typedef struct NwDefect {
    double x, y;     /* position */
    float charge;    /* +0.5 or -0.5 */
    uint32_t cells;  /* marked cells merged into this defect */
} NwDefect;
nw_status nw_find_defects(nw_system* sys, float cell_size, uint32_t flags, NwDefect* out, int max_out, int* n_out);

/* The reference's second, sampling defect search (analysis/defects.py:12-32 with
 * analysis/afa/utils.py:4-17, 35-54, analysis/afa/data.py:46-52): around each
 * sample point (the position of bead beads[k]) the beads within `radius`
 * (plain Euclidean distance, the centre bead included) are binned by the angle of
 * their displacement from the point into 8 sectors of pi/4 from -pi; a sector's
 * director is the angle of its beads' mean tangent (tangents as in
 * nw_find_defects); winding[k] = round(sum of the differences of the sector
 * directors / pi) over sectors 0 .. the highest occupied one (empty sectors read
 * 0), in float64.  The reference keeps the points with winding > 0.  One block
 * per sample point, fixed-order sums.  Synchronous.  2D systems. */
nw_status nw_sample_defects(nw_system* sys, const uint32_t* beads, int n_points, float radius, uint32_t flags,
                            int32_t* winding);

/* ---- observables ----------------------------------------------------------- */

/* Order parameters and temperatures of the current state (no counterpart in
 * the reference's step; its offline analysis defines them,
 * analysis/analyze_correlations.py:13-38 and analysis/afa/utils.py:35-49):
 *  - bead tangents as in nw_find_defects (raw differences unless
 *    NW_OBS_MIN_IMAGE; none for the first and last bead of the system);
 *  - s_q3: the largest eigenvalue of Q = 1.5 <t t> - I / 2, the mean over all
 *    beads (a bead without a tangent counts as t = 0), the reference's S;
 *  - s_2d: |<exp(2 i a)>| over the beads with a tangent, a the angle of the
 *    tangent's xy part; polar: |<t>| over all beads;
 *  - bead_temperature <m |v|^2> / dim over beads, solvent_temperature over
 *    the solvent;
 *  - msd (NW_OBS_MSD): <|r - r_ref|^2> of unwrapped bead positions since
 *    nw_observe_reset, unwrapped by the periodic images each bead crossed
 *    between calls (call at least once per half box of motion; bead indices
 *    must not move, so no filament reversal in between).
 * Fixed-order double sums.  Synchronous. */
#define NW_OBS_MIN_IMAGE 1u
#define NW_OBS_MSD 2u
typedef struct NwObservables {
    double s_q3, s_2d, polar;
    double bead_temperature, solvent_temperature;
    double msd;
    uint32_t n_beads, n_tangents, n_solvent, reserved;
} NwObservables;
nw_status nw_observe(nw_system* sys, uint32_t flags, NwObservables* out);
/* Reference positions of the mean-square displacement := the current ones. */
nw_status nw_observe_reset(nw_system* sys);
/* Velocity correlation by distance of the sampled bead pairs (d_i[k], d_j[k])
 * (device arrays of n_pairs indices): each pair's v_i . v_j enters the `bins`
 * bins of width r_max / bins by the quadratic B-spline weights of its
 * minimum-image distance (bins around its nearest bin centre, weights summing
 * to 1; the weights nwgb.observables uses), sum_dot[b] = sum w v_i . v_j,
 * sum_weight[b] = sum w (host arrays of `bins`, at most 128).  C_v(b) =
 * sum_dot / (sum_weight + 1e-3) / <|v|^2>.  Fixed-order sums.  Synchronous. */
nw_status nw_velocity_correlation(nw_system* sys, const uint32_t* d_i, const uint32_t* d_j, uint32_t n_pairs,
                                  float r_max, uint32_t bins, double* sum_dot, double* sum_weight);
/* Histogram of SRD cell temperatures sum m |v - u|^2 / (dim (n - 1)) (u the
 * cell's mass-weighted mean velocity) over the cells of two or more members
 * (beads and solvent) on the SRD grid shifted by `shift` (NULL: none):
 * counts[b] for T in [b, b + 1) t_max / bins, counts[bins] above t_max,
 * counts[bins + 1] the cells counted (host array of bins + 2).  Cell sums are
 * 2^32 fixed-point integers (independent of thread order).  Synchronous. */
nw_status nw_srd_temperature_histogram(nw_system* sys, const float shift[3], float t_max, uint32_t bins,
                                       uint32_t* counts);

/* Numerics self-check of the refined reciprocal, square root and quotient
 * the force laws use (no reference counterpart).  For host arrays a[n] and
 * b[n] of positive normal floats it writes, per element, out[4*i + 0..3] =
 * 1/a, sqrt(a), a/b computed by the device helpers, and the hardware
 * reciprocal square root of a.  Allocates and frees its own device buffers;
 * synchronous. */
nw_status nw_math_probe(const float* a, const float* b, uint32_t n, float* out);

#ifdef __cplusplus
}
#endif

#endif /* NWGB_H */
