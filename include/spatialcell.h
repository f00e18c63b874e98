/*
 * spatialcell.h -- C ABI of libspatialcell, the sm_103a (GB300) per-step
 * simulation hot path of spatial_cell_sim.
 *
 * The reference (justgos/spatial-cell, spatial_cell_sim) has no library
 * interface: its step is the body of main() (spatial_cell_sim/src/main.cu:347-700)
 * launching CUDA kernels on process-global state (__constant__ d_Config,
 * config.cuh:102).  This header is the boundary a driver binds instead:
 *
 *   reference                                     this ABI
 *   -------------------------------------------   ------------------------------
 *   Config(Json::Value)  config.cuh:46-75         sc_config, sc_config_load_json
 *   loadParticleTypeInfo chemistry.cuh:10-33      sc_types_load_json
 *   flattenParticleTypeInfo chemistry.cuh:38-51   (id-indexed sc_type_info[])
 *   loadComplexificationInfo interactions.cuh:17-54   sc_rules_load_json
 *   flattenComplexificationInfo / partnerMap...   sc_create (builds both)
 *     interactions.cuh:59-145
 *   setupParticles -> DoubleBuffer copyToDevice   sc_load_state
 *     setup/setup.cuh:17-253, memory.cuh:256
 *   initial sort + removeInterfering + complexify(-1)  sc_prepare
 *     main.cu:284-338
 *   one iteration of the step loop main.cu:347-661    sc_step
 *   single kernels of that loop                   sc_run_phase
 *   reduceParticles + persistFrame                sc_reduce_frame
 *     dynamics.cuh:824-844, main.cu:95-126
 *   FileStorage writeHeader / writeFrame          sc_frames_write_header / _frame
 *     storage.cuh:22-39
 *
 * Conventions: every function returns 0 on success and a negative SC_E_*
 * code on failure; sc_last_error() gives the message.  A sim owns all of its
 * device memory and one CUDA stream; calls on one sim must come from one host
 * thread at a time, different sims are independent.  Layouts below are the
 * reference's structs byte for byte (types.cuh:167-300, NUM_METABOLITES = 10).
 */
#ifndef SPATIALCELL_H
#define SPATIALCELL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SC_MAX_ACTIVE_INTERACTIONS 8  /* constants.cuh:18 */
#define SC_AOS_NUM_METABOLITES 10     /* constants.cuh:15 */
#define SC_REDUCED_NUM_METABOLITES 4  /* constants.cuh:16 */
#define SC_PARTICLE_FLAG_ACTIVE 0x1   /* constants.cuh:23 */
#define SC_INTERACTION_TYPE_CHAIN 1
#define SC_INTERACTION_GROUP_FORWARD 10
#define SC_INTERACTION_GROUP_BACKWARD 11
#define SC_PARTICLE_TYPE_LIPID 0
#define SC_PARTICLE_TYPE_METABOLIC 1000
#define SC_HYDROPHYLIC 0
#define SC_HYDROPHOBIC 1
#define SC_POLAR 2

/* Status codes */
#define SC_OK 0
#define SC_E_INVALID (-1)  /* bad argument, config or table */
#define SC_E_CUDA (-2)     /* CUDA runtime error */
#define SC_E_OOM (-3)      /* device allocation failed */
#define SC_E_IO (-4)       /* file open / read / write failed */
#define SC_E_PARSE (-5)    /* malformed JSON */
#define SC_E_DEVICE (-6)   /* a kernel reported an error (bounded wait expired, bounds) */
#define SC_E_STATE (-7)    /* call out of order (e.g. step before load) */

/* ParticleInteraction, types.cuh:167-171 (12 bytes) */
typedef struct sc_interaction {
    int32_t type;
    int32_t group;
    int32_t partner_id;
} sc_interaction;

/* Particle, types.cuh:173-222 (256 bytes). */
typedef struct sc_particle {
    int32_t id;                        /*   0 */
    int32_t type;                      /*   4 */
    int32_t flags;                     /*   8 */
    int8_t state;                      /*  12 */
    int8_t _pad0[3];
    int32_t last_state_change_step;    /*  16 */
    float radius;                      /*  20 */
    int8_t hydrophobic;                /*  24 */
    int8_t _pad1[3];
    float pos[3];                      /*  28 */
    float _pad2[2];
    float rot[4];                      /*  48 */
    float velocity[3];                 /*  64 */
    float pos_noise[3];                /*  76 */
    float _pad3[2];
    float angular_velocity[4];         /*  96 */
    float angular_noise[4];            /* 112 */
    int32_t n_active_interactions;     /* 128 */
    sc_interaction interactions[SC_MAX_ACTIVE_INTERACTIONS]; /* 132 */
    int32_t scheduled_polymerization;  /* 228 */
    float _pad4[2];
    float debug_vector[4];             /* 240 */
} sc_particle;

/* MetabolicParticle, types.cuh:224-242 (304 bytes). */
typedef struct sc_metabolic_particle {
    sc_particle p;                               /*   0 */
    float metabolites[SC_AOS_NUM_METABOLITES];   /* 256 */
    float _pad[2];
} sc_metabolic_particle;

/* ReducedParticle, types.cuh:244-287 (36 bytes); halves are IEEE binary16. */
typedef struct sc_reduced_particle {
    int32_t id;
    int32_t type;
    int32_t flags;        /* flags | (state & 0xF) << 16 */
    uint16_t radius;
    uint16_t pos[3];
    uint16_t rot[4];
    uint16_t debug_vector[4];
} sc_reduced_particle;

/* ReducedMetabolicParticle, types.cuh:289-300 (44 bytes). */
typedef struct sc_reduced_metabolic_particle {
    sc_reduced_particle p;
    uint16_t metabolites[SC_REDUCED_NUM_METABOLITES];
} sc_reduced_metabolic_particle;

/* MinimalParticleTypeInfo, types.cuh:16-32 (8 bytes); id-indexed table. */
typedef struct sc_type_info {
    float radius;
    int8_t hydrophobic;
    int8_t _pad[3];
} sc_type_info;

/* ParticleInteractionInfo, types.cuh:55-126 (96 bytes). */
typedef struct sc_rule {
    int32_t id;                          /*  0 */
    int32_t group;                       /*  4 */
    int32_t first_partner_type;          /*  8 */
    int8_t first_partner_state;          /* 12 */
    int8_t _pad0[3];
    int32_t second_partner_type;         /* 16 */
    int8_t second_partner_state;         /* 20 */
    uint8_t propagate_state;             /* 21 */
    uint8_t set_state;                   /* 22 */
    uint8_t wait_for_state;              /* 23 */
    uint8_t wait_for_alignment;          /* 24 */
    uint8_t only_via_transition;         /* 25 */
    uint8_t _pad1[2];
    int32_t transition_to;               /* 28 */
    int32_t polymerize;                  /* 32 */
    uint8_t break_after_transition;      /* 36 */
    /* extension, in the reference struct's padding (honoured only by sims
       created with sc_config.rule_probabilities = 1): when use_probability
       is set, complexify forms a bond under this rule only with the given
       probability per step, drawn from Philox keyed by (seed, rule id, step,
       lower id, higher id) so both partners draw the same number
       (complexification.json key "probability") */
    uint8_t use_probability;             /* 37 */
    uint8_t _pad2[10];
    float relative_orientation[4];       /* 48 */
    float orientation_alignment_threshold; /* 64 */
    float relative_position[3];          /* 68 */
    float position_alignment_threshold;  /* 80 */
    float probability;                   /* 84 (extension, see use_probability) */
    float _pad3[2];
} sc_rule;

/* config.json (spatial_cell_sim/config.json, config.cuh:15-75) plus
 * extension keys whose defaults reproduce the reference. */
typedef struct sc_config {
    int32_t num_particles;            /* particle capacity */
    int32_t num_metabolic_particles;  /* metabolic particle capacity */
    int32_t steps;
    float sim_size;
    float max_interaction_distance;
    float max_diffusion_distance;
    float grid_cell_size;
    float movement_noise_scale;
    float rotation_noise_scale;
    float metabolite_movement_noise_scale;
    float velocity_decay;
    float angular_velocity_decay;
    int32_t noise_coordination_steps;
    int32_t relaxation_steps;
    int32_t metabolite_diffusion_steps;
    int32_t persist_every_nth_frame;
    int32_t report_every_nth_frame;
    /* extensions */
    int32_t num_metabolites;  /* simulated species S, 1..10 (reference: 10) */
    int32_t periodic;         /* 0: the reference's walls (positions clamped to
                                 [0, simSize]); 1: periodic box (minimum-image
                                 pairs, wrapped cells and positions; needs at
                                 least 3 cells per axis) */
    int32_t walls;            /* walled box (periodic = 0): 0 the reference's clamp of
                                 positions to [0, simSize]; 1 reflecting walls (a step
                                 past a wall is mirrored back into the box) */
    uint64_t seed;            /* Philox key of the Brownian noise */
    /* execution switches of one sim (results do not depend on them; the
       values of sc_config_defaults are the production settings) */
    int32_t graphs;           /* 1: each step replayed as a captured CUDA graph; 0: launched
                                 phase by phase */
    int32_t class_streams;    /* particle relax work classes: 0 chosen by size (three streams
                                 when the particles fill the device), 1 on the sim's stream,
                                 3 on three streams */
    int32_t tiles;            /* metabolic sweeps: 0 per-item pair lists, 1 shared-memory tiles */
    int32_t pair_list_limit;  /* -1: pair lists at full capacity; n >= 0: at most n entries per
                                 list (the items beyond take the neighbourhood-scan paths) */
    int32_t pool_per_item;    /* -1: the metabolic pair pool is sized by the scene's demand at
                                 sc_prepare; n >= 0: it starts at n entries per metabolic item
                                 (it grows to its demand at the next synchronisation either way) */
    /* complexify extension: 0 the reference's per-item scan (every passing
       rule appends a bond on the scanning item's side); 1 deterministic pair
       claim: every item offers itself to each neighbour that passes a rule's
       gates with the 64-bit key (distance bits, item slot) by atomicMin, and
       two items bond only when each holds the other's key -- at most one new
       rule bond per item per step, always on both sides */
    int32_t pair_claim;
    /* 1: honour the probability extension of the rule records
       (sc_rule.use_probability / probability); 0: ignore those bytes, which
       are padding in the reference's own records and may hold anything */
    int32_t rule_probabilities;
    /* metabolic relaxation pairs: 1 (default) a 16-byte entry per pair with
       the pair's position-only term evaluated once per step; 0 a 4-byte
       entry (the neighbour), the term evaluated again in each sub-iteration
       (a quarter of the pool's memory, about twice the sweep's time) */
    int32_t metabolic_pairs;
    /* 1: after polymerize, each particle takes the state (and its last
       state-change step) of a bonded partner whose state changed later, over
       the bonds whose rule sets propagateState -- the reference's
       propagateState kernel (interactions.cuh:743-822), which its step
       leaves commented out (main.cu:618-631); 0 (default): the reference's
       step, without it */
    int32_t propagate_state;
    int32_t _reserved;
} sc_config;

/* Counters of a sim (the reference's nActiveParticles, lastActiveParticle,
 * nextParticleId and nActiveMetabolicParticles buffers, main.cu:244-253). */
typedef struct sc_counters {
    int32_t n_active_particles;
    int32_t n_active_metabolic_particles;
    int32_t next_particle_id;
    int32_t step;
    int64_t kernel_launches;   /* kernels this sim has launched so far */
    int32_t device_error;      /* sticky kernel-side error code, 0 if none */
    int32_t _reserved;
} sc_counters;

/* Phases for sc_run_phase: one reference kernel (or kernel pair) each. */
enum sc_phase {
    SC_PHASE_SORT_PARTICLES = 0,      /* updateGridAndSort<Particle>, grid.cuh:111-139 */
    SC_PHASE_SORT_METABOLIC = 1,      /* updateGridAndSort<MetabolicParticle> */
    SC_PHASE_MOVE_BROWNIAN = 2,       /* move + brownianMovementAndRotation<Particle>, main.cu:375-395 */
    SC_PHASE_MOVE_BROWNIAN_METAB = 3, /* moveMetabolicParticles + brownian<Metabolic>, main.cu:402-419 */
    SC_PHASE_COORDINATE_NOISE = 4,    /* coordinateNoise, fraction = arg / noiseCoordinationSteps */
    SC_PHASE_APPLY_NOISE = 5,         /* applyNoise<Particle> + applyNoise<Metabolic> */
    SC_PHASE_RELAX = 6,               /* relax, dynamics.cuh:405-822 */
    SC_PHASE_RELAX_METAB = 7,         /* relaxMetabolicParticles, metabolites.cuh:140-264 */
    SC_PHASE_RELAX_PARTNERS = 8,      /* relaxMetabolicParticlePartners, metabolites.cuh:266-350 */
    SC_PHASE_APPLY_VELOCITIES = 9,    /* applyVelocities x2 (fraction 0.45) */
    SC_PHASE_COMPLEXIFY = 10,         /* complexify, interactions.cuh:216-346 */
    SC_PHASE_TRANSITION = 11,         /* transitionInteractions, interactions.cuh:349-555 */
    SC_PHASE_POLYMERIZE = 12,         /* polymerize, interactions.cuh:558-740 */
    SC_PHASE_DIFFUSE = 13,            /* diffuseMetabolites, metabolites.cuh:352-431 */
    SC_PHASE_REMOVE_INTERFERING = 14, /* removeInterferingMetabolicParticles, metabolites.cuh:18-88 */
    SC_PHASE_END_STEP = 15,           /* step counter += 1 */
    SC_PHASE_PROPAGATE_STATE = 16     /* propagateState, interactions.cuh:743-822 (sc_config.propagate_state) */
};

typedef struct sc_sim sc_sim;

/* ---- configuration and tables (host only) ---- */
/* Reference defaults (spatial_cell_sim/config.json) plus extension defaults. */
void sc_config_defaults(sc_config *cfg);
/* Parses config.json (Config(Json::Value), config.cuh:46-64).  Missing keys
 * keep the values already in *cfg. */
int sc_config_load_json(const char *path, sc_config *cfg);
/* Derived grid values of config.cuh:65-74 (cells per axis rounded up to a
 * power of two, at least 2). */
int sc_config_grid(const sc_config *cfg, int32_t *n_grid_cells, int32_t *n_grid_bits);
/* large-molecules.json -> id-indexed table (chemistry.cuh:10-51).  Writes
 * max(type)+1 entries (missing ids zero) if they fit in capacity; *n_types
 * always receives the required count. */
int sc_types_load_json(const char *path, sc_type_info *out, int32_t capacity, int32_t *n_types);
/* complexification.json -> rule list in file order (interactions.cuh:17-54),
 * with jsoncpp's defaults and its null handling (an explicit null reads as 0). */
int sc_rules_load_json(const char *path, sc_rule *out, int32_t capacity, int32_t *n_rules);

/* ---- simulation ---- */
/* Creates a sim on the current CUDA device.  types: id-indexed, n_types
 * entries.  rules: any order; the first of duplicate ids wins. */
int sc_create(const sc_config *cfg, const sc_type_info *types, int32_t n_types,
              const sc_rule *rules, int32_t n_rules, sc_sim **out);
void sc_destroy(sc_sim *sim);
/* Message of the last failure of this sim (sim == NULL: of the last failed
 * call that had no sim). */
const char *sc_last_error(const sc_sim *sim);

/* Uploads a reference-layout state.  particles[0..n) and metabolic[0..nm) are
 * the set-up items; the rest of capacity is zero (inactive), as the
 * reference's memset host buffers are.  n and nm become the active counters
 * (nActiveParticles, nActiveMetabolicParticles); step is the loop counter of
 * the next step; next_particle_id the id the next polymerised monomer gets. */
int sc_load_state(sc_sim *sim, const sc_particle *particles, int32_t n,
                  const sc_metabolic_particle *metabolic, int32_t nm,
                  int32_t step, int32_t next_particle_id);
/* main.cu:284-338: sort both sets, removeInterferingMetabolicParticles, and
 * the initial complexify (step -1). */
int sc_prepare(sc_sim *sim);
/* Runs n_steps iterations of the step loop (main.cu:347-661) asynchronously
 * on the sim's stream. */
int sc_step(sc_sim *sim, int32_t n_steps);
/* Runs one phase of the loop (for differential testing). */
int sc_run_phase(sc_sim *sim, int32_t phase, int32_t arg);
/* Waits for the sim's stream and reports kernel-side errors. */
int sc_sync(sc_sim *sim);
/* Pairs held by the current pair lists (no counterpart in the reference; for
 * measurement): out[0] particle pairs (coordinateNoise / relax), out[1]
 * metabolic relaxation, out[2] lipid-metabolic, out[3] diffusion; -1 for a
 * list not built since its inputs last changed.  Waits for the sim. */
int sc_pair_counts(sc_sim *sim, int64_t out[4]);
/* Items whose pair list overflowed its capacity (they take the scan paths),
 * per list in the order of sc_pair_counts; -1 for a list not built since its
 * inputs last changed.  Waits for the sim. */
int sc_list_overflows(sc_sim *sim, int64_t out[4]);
/* 1 when all work enqueued on the sim has finished, 0 while some is still
 * running (does not wait; for loops that drive many sims at once). */
int sc_idle(sc_sim *sim);

/* Downloads the state in the reference layout, capacity-sized buffers (either
 * may be NULL).  Interaction slots at and beyond n_active_interactions are
 * written as zero. */
int sc_export_state(sc_sim *sim, sc_particle *particles, sc_metabolic_particle *metabolic);
/* Sort results of the last sort: which = 0 particles, 1 metabolic.
 * ranges: 2 * cells uint32 in the reference's gridRanges layout ([start, end)
 * per cell, zero for empty cells); perm: capacity entries, the pre-sort slot
 * of every sorted slot.  Either may be NULL. */
int sc_export_grid(sc_sim *sim, int32_t which, uint32_t *ranges, uint32_t *perm);
int sc_get_counters(sc_sim *sim, sc_counters *out);
/* The sim's CUDA stream (a cudaStream_t), for callers that order their own
 * work or timing events after the sim's. */
void *sc_get_stream(sc_sim *sim);
/* Completion notices (no counterpart in the reference; for loops that
 * drive many sims at once without polling them).  With a key set (>= 0),
 * every sc_step call of the sim queues the key once the work it enqueued has
 * finished on the device; sc_wait_notices blocks until at least one key is
 * queued or timeout_ms has passed (< 0: no limit, 0: does not wait), takes up
 * to cap keys in the order they were queued, and returns how many it took.
 * The queue is shared by every sim of the process. */
int sc_set_notify(sc_sim *sim, int64_t key);
int32_t sc_wait_notices(int64_t *keys, int32_t cap, int32_t timeout_ms);
/* Device memory the sim holds now, in bytes (no counterpart in the
 * reference; for admission against a memory budget). */
int sc_device_bytes(const sc_sim *sim, int64_t *bytes);
/* The frames.dat payload of the current state (reduceParticles on the
 * counters' ranges, zero beyond), into capacity-sized host buffers. */
int sc_reduce_frame(sc_sim *sim, sc_reduced_particle *particles,
                    sc_reduced_metabolic_particle *metabolic);
/* The same frame, streamed: the reduction is enqueued on the sim's stream
 * behind the work already there and the copy to the host runs on a second
 * stream, so the steps enqueued next overlap it (the reference hands each
 * frame to a std::async writer thread, main.cu:95-126).  Two frames can be in
 * flight; a third waits on the device for the first one's copy.  The host
 * buffers must stay valid until the frame has landed, and must be pinned
 * (cudaHostAlloc / cudaHostRegister) for the copy to overlap the steps.
 * Returns the frame's ticket (>= 0) or a negative SC_E_* code. */
int64_t sc_reduce_frame_async(sc_sim *sim, sc_reduced_particle *particles,
                              sc_reduced_metabolic_particle *metabolic);
/* Blocks until frame `ticket` (and every earlier frame) is in host memory. */
int sc_frame_wait(sc_sim *sim, int64_t ticket);

/* ---- batched replicas (no counterpart in the reference) ----
 * One sim that steps many independent replica cells together: every phase
 * is one launch over the items of all replicas, the sort orders one key
 * space in which each replica's cells follow the previous replica's (the
 * replica in the key's high part), and each kernel works on an item with
 * its replica's box, cells and noise key.  A replica evolves exactly as a
 * sim of its own created with the same config, box, capacities and seed,
 * bit for bit.  The config gives the shared physics (noise scales, ranges,
 * cell size, sub-iterations, box kind, extension switches); its capacities
 * and box are replaced by the replicas'.  Rules that polymerise are not
 * accepted, and the sim-wide calls that need one box (sc_generate_*,
 * sc_mark_positions, sc_observe, sc_pair_histogram, sc_checkpoint_*) return
 * SC_E_INVALID on a batch; sc_step, sc_run_phase, sc_sync, sc_reduce_frame
 * (records of all replicas in slot order) and sc_export_grid work as for
 * any sim. */
typedef struct sc_replica {
    int32_t num_particles;            /* the replica's particle capacity */
    int32_t num_metabolic_particles;  /* its metabolic capacity */
    float sim_size;                   /* its box */
    int32_t _pad;
    uint64_t seed;                    /* Philox key of its noise */
} sc_replica;
int sc_create_batch(const sc_config *cfg, const sc_replica *replicas, int32_t n_replicas, const sc_type_info *types,
                    int32_t n_types, const sc_rule *rules, int32_t n_rules, sc_sim **out);
/* Loads the replicas' states: particles / metabolic hold replica 0's
 * n[0] / nm[0] records, then replica 1's, and so on (the layout of
 * sc_load_state per replica). */
int sc_load_batch(sc_sim *sim, const sc_particle *particles, const int32_t *n, const sc_metabolic_particle *metabolic,
                  const int32_t *nm, int32_t step);
/* Fills every replica on the device: replica r gets the scene
 * sc_generate_uniform(n[r], nm[r], kinds, fractions + r * nkinds, nkinds,
 * seeds[r]) writes for a sim of its own with the replica's box. */
int sc_generate_batch(sc_sim *sim, const int32_t *n, const int32_t *nm, const int32_t *kinds, const float *fractions,
                      int32_t nkinds, const uint64_t *seeds);
/* Replica r's records in slot order into buffers of its capacities (zero
 * past its records): what sc_export_state gives for a sim of its own. */
int sc_export_replica(sc_sim *sim, int32_t replica, sc_particle *particles, sc_metabolic_particle *metabolic);

/* ---- allocation-free cell sort (no counterpart in the reference) ----
 * For callers that cannot let a library allocate device memory: a framework
 * that owns the GPU's memory as its own pool, or a loop that cannot absorb
 * the device-wide synchronisation of cudaMalloc / cudaFree.  Runs the binning
 * of a sim's sort -- cell key of every item, stable onesweep radix sort, cell
 * start table -- on buffers the caller owns; its working memory is one fixed
 * static device array inside the library.
 *   pos:  n float4 (x, y, z, radius), device memory
 *   info: n int4 (id, type, flags, hydrophobic); only bit 0 of flags (active)
 *         is read; device memory
 *   perm: n uint32 out, the input index of every sorted slot
 *   cell_start: cells + 1 uint32 out, cells = n_grid_cells^3 (sc_config_grid):
 *         first sorted slot of every cell (a cell's items are
 *         [cell_start[c], cell_start[c + 1]); inactive items come last)
 *   stream: a cudaStream_t (NULL: the legacy default stream)
 * Limit: n <= 262144; larger n returns SC_E_INVALID and launches nothing.
 * The static array (about 4.3 MB) stays on every GPU that loads the library
 * until the process exits.  All calls on a GPU share it, so calls whose work
 * overlaps on that GPU race; order them on one stream.  Every call looks up
 * the array's address on the current device (no allocation) and waits for
 * its own results: it returns once they are in perm / cell_start, so it is
 * synchronous and cannot be made while the stream is being captured.
 * SC_E_DEVICE if the sort reported an error. */
int sc_sort_cells_static(const sc_config *cfg, const void *pos, const void *info, int32_t n, uint32_t *perm,
                         uint32_t *cell_start, void *stream);

/* ---- device scene generation (no counterpart in the reference) ----
 * Replaces host-side uniform scene setup (setup/particle_setup.cuh) for
 * callers that create many sims: fills the sim on the device with n
 * particles (kind k of kinds[] with probability fractions[k], k < nkinds <= 4,
 * position uniform in the box, uniform random orientation) and nm metabolic
 * particles (type 1000, uniform, species 0 seeded at 100 in x < 0.2 * box,
 * the other species uniform in [0, 10)), every record a function of (seed,
 * index) only; radii and hydrophobicity come from the sim's type table.
 * Counters as sc_load_state with step 0 and next particle id n. */
int sc_generate_uniform(sc_sim *sim, int32_t n, int32_t nm, const int32_t *kinds, const float *fractions,
                        int32_t nkinds, uint64_t seed);

/* Structured scenes: the particles are a list of groups, generated on the
 * device one after another (group g's particles follow group g-1's; ids are
 * indices), the metabolic particles as in sc_generate_uniform.  Group kinds
 * restate the reference's host setup helpers (setup/particle_setup.cuh,
 * setup/interaction_setup.cuh) with counter-based draws in place of its
 * std::mt19937 stream:
 *   UNIFORM_BOX      count particles uniform in the box (fillParticlesUniform)
 *   UNIFORM_BALL     count particles uniform in the ball (center, radius)
 *   SPHERE_SHELL     count particles uniform on the sphere (center, radius),
 *                    oriented quaternionFromTo(up, radial) * rot as
 *                    fillParticlesSphere orients them
 *   FIBONACCI_SHELL  fillParticlesSphere: count points of the Fibonacci
 *                    spiral on the sphere; radius <= 0 takes the
 *                    reference's count-based radius
 *   COMPLEXES        count complexes of unit particles on a random patch of
 *                    the cubic lattice of the given spacing (grown site by
 *                    site from a neighbour of an earlier site), one random
 *                    orientation per complex, centre uniform in the ball;
 *                    each site bonded to the site it grew from
 *   WRAPPED_CHAINS   count chains of unit particles (fillParticlesWrappedChain,
 *                    each member's step -(radius of type id t-1 + radius of
 *                    t) along its up vector, its orientation slerped 0.3 of
 *                    the way to a random one), start uniform in the ball,
 *                    linked serially (linkParticlesSerially)
 * Member types are drawn from the group's mix (kinds / fractions), except
 * chains, whose member k has kind k % nkinds.  Bonds use interaction type
 * link_type with group FORWARD on the earlier particle and BACKWARD on the
 * later one.  Positions are clamped into [0, sim_size] as the reference's
 * helpers clamp them. */
#define SC_SCENE_UNIFORM_BOX 0
#define SC_SCENE_UNIFORM_BALL 1
#define SC_SCENE_SPHERE_SHELL 2
#define SC_SCENE_FIBONACCI_SHELL 3
#define SC_SCENE_COMPLEXES 4
#define SC_SCENE_WRAPPED_CHAINS 5
#define SC_SCENE_MAX_UNIT 64

typedef struct sc_scene_group {
    int32_t kind;          /* SC_SCENE_* */
    int32_t count;         /* particles, or complexes / chains */
    int32_t unit;          /* particles per complex / chain (<= SC_SCENE_MAX_UNIT) */
    int32_t nkinds;        /* 1 .. 4 */
    int32_t kinds[4];      /* type ids */
    float fractions[4];    /* relative weights */
    float center[3];
    float radius;          /* ball / sphere radius */
    float spacing;         /* complex lattice spacing */
    float rot[4];          /* shells: base orientation (x, y, z, w) */
    int32_t link_type;     /* interaction type of complex / chain bonds */
} sc_scene_group;

/* Fills the sim with the groups' particles (their total must fit its
 * capacity) and nm metabolic particles; counters as sc_generate_uniform. */
int sc_generate_scene(sc_sim *sim, const sc_scene_group *groups, int32_t n_groups, int32_t nm, uint64_t seed);
/* Batched sims: every replica r gets the groups' particles and nm metabolic
 * particles as sc_generate_scene with seeds[r] gives a sim of its own (the
 * groups' coordinates are the same in every replica's box); the replicas'
 * particle and metabolic capacities must hold them.  Records are generated
 * one replica at a time, so the staging memory is one replica's. */
int sc_generate_scene_batch(sc_sim *sim, const sc_scene_group *groups, int32_t n_groups, int32_t nm,
                            const uint64_t *seeds);

/* ---- observables (no counterpart in the reference) ----
 * Ensemble quantities reduced on the device in double precision, in a fixed
 * order (the same bytes on every run).  Index 0 is the particles, 1 the
 * metabolic particles; only active items count. */
typedef struct sc_observables {
    double msd[2];            /* mean squared displacement since sc_mark_positions (nm^2), items
                                 matched by id; minimum image in a periodic box */
    int64_t msd_items[2];     /* items in the mean (active, with a mark) */
    double mean_v2[2];        /* mean |velocity|^2 */
    int64_t active[2];        /* active items */
    int64_t bond_slots;       /* sum of n_active_interactions over active particles */
    double metabolites[SC_AOS_NUM_METABOLITES]; /* total amount of each simulated species */
} sc_observables;
/* Records every active item's position, by id, as the origin of the MSD. */
int sc_mark_positions(sc_sim *sim);
int sc_observe(sc_sim *sim, sc_observables *out);
/* Histogram of the distances of ordered particle pairs (i, j), i != j, i of
 * type type_a and j of type type_b (-1: any type), active, closer than r_max
 * (at most the grid cell size): counts[b] for distance in
 * [b, b + 1) * r_max / n_bins.  Distances in double precision from the float
 * positions (minimum image in a periodic box).  Sorts the particles into
 * their cells first when they have moved since the last sort (the next
 * step's sort then leaves them in place, so the trajectory is unchanged). */
int sc_pair_histogram(sc_sim *sim, int32_t type_a, int32_t type_b, float r_max, int32_t n_bins, uint64_t *counts);

/* ---- checkpoint / resume (no counterpart in the reference) ----
 * A checkpoint holds the whole state -- the active particle and metabolic
 * records in the reference's layouts, the step counter and the next particle
 * id -- after a 24-byte header: "SCCKPT01", then the particle and metabolic
 * record counts, the step and the next particle id as int32.  Reading it into a sim created with the same configuration and
 * tables and calling sc_step continues the run bit for bit: noise is keyed by
 * (seed, particle id, step) and every pair list is rebuilt.  `file` is a
 * FILE* open for binary writing / reading. */
int sc_checkpoint_write(sc_sim *sim, void *file);
int sc_checkpoint_read(sc_sim *sim, void *file);

/* ---- frames.dat (storage.cuh:9-44) ---- */
int sc_frames_write_header(void *file /* FILE* */, const sc_config *cfg);
int sc_frames_write_frame(void *file /* FILE* */, const sc_config *cfg,
                          const sc_reduced_particle *particles,
                          const sc_reduced_metabolic_particle *metabolic);

#ifdef __cplusplus
}
#endif

#endif /* SPATIALCELL_H */
