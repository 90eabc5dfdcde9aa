/*
 * lpg.h — C ABI of the GB300 per-tick agent step for laser-polio models.
 *
 * The reference (laser_polio, pure Python + numba) has no native ABI: its
 * per-tick path is the SEIR_ABM tick loop (laser_polio/model.py:246-282)
 * calling each component's step() and log() over host numpy columns.  The
 * entry points below are what those component classes call instead; each
 * comment names the reference code it replaces.  Everything crosses this
 * boundary as plain pointers and sizes: no torch, no CUDA types.
 *
 * Conventions
 *   - Every function returns LPG_OK (0) or a negative lpg_status.  The text
 *     of the last error is available from lpg_last_error().
 *   - One handle holds one or more simulations ("replicates") that advance
 *     in lockstep on one GPU and one CUDA stream.  A handle is not
 *     thread-safe; calls on one handle must be serialized.
 *   - Agent columns are passed in the reference's slot order
 *     (LaserFrame index order, laser_polio/model.py:139-172), length
 *     `capacity`.  Pointers may be host or device memory (CUDA unified
 *     addressing decides); NULL means "column absent, use the reference's
 *     default".
 *   - Result arrays are int32, row-major [nt][n_nodes] or
 *     [nt][n_nodes][n_strains], exactly the shapes of sim.results
 *     (laser_polio/model.py:548-559, 1216, 1267-1272, 1601-1602, 1898-1917,
 *     2086-2092).
 */
#ifndef LPG_H
#define LPG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LPG_ABI_VERSION 1
#define LPG_MAX_STRAINS 4
#define LPG_MAX_SIA_PER_DAY 8

typedef enum {
  LPG_OK = 0,
  LPG_ERR_ARG = -1,      /* bad argument (sizes, pointers, parameter ranges) */
  LPG_ERR_CAPACITY = -2, /* births exceed capacity (LaserFrame.add, model.py:1719) */
  LPG_ERR_NODE = -3,     /* node id outside [0, n_nodes) */
  LPG_ERR_TIMEOUT = -4,  /* a bounded device loop gave up */
  LPG_ERR_CUDA = -5,     /* CUDA runtime error */
  LPG_ERR_STATE = -6,    /* call out of order (e.g. step before start) */
  LPG_ERR_NOMEM = -7,    /* device allocation failed */
  LPG_ERR_INTERNAL = -8  /* an internal consistency check failed */
} lpg_status;

/* Component mask: which of the five reference components are present
 * (SEIR_ABM.components, laser_polio/model.py:209-244). */
enum {
  LPG_COMP_VD = 1,  /* VitalDynamics_ABM  model.py:1521-1765 */
  LPG_COMP_DS = 2,  /* DiseaseState_ABM   model.py:505-812   */
  LPG_COMP_RI = 4,  /* RI_ABM             model.py:1858-1992 */
  LPG_COMP_SIA = 8, /* SIA_ABM            model.py:2063-2163 */
  LPG_COMP_TX = 16  /* Transmission_ABM   model.py:1152-1491 */
};

/* A Distribution (laser_polio/distributions.py:17-102): kind is one of
 * LPG_DIST_* in the engine headers: 0 constant(value), 1 exponential(scale),
 * 2 gamma(shape, scale), 3 lognormal(mean, sigma), 4 normal(mean, std),
 * 5 poisson(lam), 6 uniform(min, max), 7 lognormal_int(mean, sigma). */
typedef struct {
  int32_t kind;
  double p1, p2;
} lpg_dist;

/* One SIA campaign (SIA_ABM.step, model.py:2099-2156), already resolved to
 * the tick on which the reference would run it. */
typedef struct {
  int32_t tick;
  int32_t strain;           /* vaccine strain (model.py:2115-2120) */
  int32_t min_age, max_age; /* inclusive window in days (model.py:2042) */
  double efficacy;          /* pars.vx_efficacy[vaccinetype] */
  const uint8_t* node_mask; /* [n_nodes], nonzero = node targeted */
} lpg_sia_event;

/* One seed_schedule entry (DiseaseState_ABM.step, model.py:759-786). */
typedef struct {
  int32_t tick;
  int32_t node;
  int32_t is_count; /* 1: value is a head count; 0: value is a prevalence fraction */
  double value;
} lpg_seed_event;

/* Everything one simulation needs besides its agent columns.  All pointers
 * are host pointers and are copied by lpg_create. */
typedef struct {
  int32_t n_nodes;
  int32_t n_strains; /* len(pars.strain_ids), <= LPG_MAX_STRAINS */
  int32_t nt;        /* pars.dur + 1 */
  int64_t count;     /* people.count at the start */
  int64_t capacity;  /* people.capacity */
  uint64_t seed;     /* keys the counter-based draws */
  uint32_t components;
  int32_t stop_if_no_cases;

  /* VitalDynamics_ABM */
  int32_t vd_step;               /* pars.step_size_VitalDynamics_ABM */
  const double* birth_rate;      /* [n_nodes] cbr / 365000 (model.py:1669-1675) */
  const int64_t* km_cumdeaths;   /* cumulative deaths by age-year (utils.py:795-816) */
  int32_t km_len;                /* entries in km_cumdeaths */
  int32_t km_max_year;           /* max_year of predict_age_at_death */

  /* DiseaseState_ABM */
  float p_paralysis;
  const lpg_seed_event* seeds;
  int32_t n_seeds;
  lpg_dist dur_inf;              /* used to redraw timers of seeded agents */

  /* RI_ABM */
  int32_t ri_step;               /* pars.step_size_RI_ABM */
  int32_t ri_enabled;            /* 0 when pars.vx_prob_ri is None */
  int32_t ri_strain;             /* model.py:1934-1940 */
  const double* vx_prob_ri;      /* [n_nodes] */
  const double* vx_prob_ipv;     /* [n_nodes] */

  /* SIA_ABM */
  const lpg_sia_event* sia;
  int32_t n_sia;
  const float* vx_prob_sia;      /* [n_nodes] float32 (model.py:2109) */

  /* Transmission_ABM */
  const double* strain_r0_scalars; /* [n_strains] */
  const double* network;           /* [n_nodes][n_nodes], network[i][j] = flow i->j */
  const double* r0_scalars;        /* [n_nodes] */
  const double* seasonality;       /* [nt] get_seasonality at each tick (utils.py:616-625) */
  double zero_inflation;           /* pars.node_seeding_zero_inflation */
  int32_t nb_r;                    /* max(1, round(pars.node_seeding_dispersion)) */

  /* results present before the first tick */
  const int32_t* pop0;             /* [n_nodes] results.pop[0] (model.py:559) */
  const int32_t* R_preseed;        /* [nt][n_nodes] added into results.R, or NULL */
} lpg_sim_desc;

/* Agent columns (LaserFrame properties), reference slot order, length
 * capacity.  Element types are those of the reference. */
typedef struct {
  int8_t* disease_state;         /* model.py:144 */
  int8_t* strain;                /* model.py:151 */
  int8_t* exposure_timer;        /* model.py:571 */
  int8_t* infection_timer;       /* model.py:572 */
  int8_t* paralysis_timer;       /* model.py:573 */
  int8_t* potentially_paralyzed; /* model.py:146 */
  int8_t* paralyzed;             /* model.py:149 */
  int8_t* ipv_protected;         /* model.py:150 */
  uint8_t* chronically_missed;   /* model.py:153 */
  int16_t* node_id;              /* model.py:161 */
  int16_t* ri_timer;             /* model.py:1891 */
  float* acq_risk_multiplier;    /* model.py:1201 */
  float* daily_infectivity;      /* model.py:1204 */
  int32_t* date_of_birth;        /* model.py:1550 */
  int32_t* date_of_death;        /* model.py:1603 */
} lpg_columns;

/* Result arrays to fill; NULL entries are skipped. */
typedef struct {
  int32_t* S;
  int32_t* E;
  int32_t* I;
  int32_t* R;
  int32_t* E_by_strain;
  int32_t* I_by_strain;
  int32_t* potentially_paralyzed;
  int32_t* paralyzed;
  int32_t* new_potentially_paralyzed;
  int32_t* new_paralyzed;
  int32_t* pop;
  int32_t* births;
  int32_t* deaths;
  int32_t* new_exposed;
  int32_t* new_exposed_by_strain;
  int32_t* ri_vaccinated;
  int32_t* ri_protected;
  int32_t* ri_new_exposed_by_strain;
  int32_t* ipv_vaccinated;
  int32_t* sia_vaccinated;
  int32_t* sia_protected;
  int32_t* sia_new_exposed_by_strain;
} lpg_results_view;

typedef struct {
  int32_t t;       /* next tick to run (SEIR_ABM.t) */
  int32_t stopped; /* early stop fired (SEIR_ABM.should_stop) */
  int64_t count;   /* people.count */
  int32_t error;   /* sticky device-side error (lpg_status), 0 if none */
} lpg_sim_state;

/* Per-kernel device time accumulated while profiling is on. */
typedef struct {
  int32_t n_kernels;
  const char* names[16];
  double total_ms[16];
  int64_t launches[16];
} lpg_profile;

typedef struct lpg_handle lpg_handle;

/* Library version and the name of the device code it carries. */
int lpg_version(void);

/* Every check lpg_create makes on one simulation's description (sizes,
 * required arrays, event ranges, and that the parameter arrays are finite
 * and in range, where the reference raises ValueError: model.py:169-170,
 * 602, 687, 702, 770, 1256), on the host, without a GPU.  LPG_OK or the
 * status lpg_create would return; the text from lpg_op_last_error().  A
 * caller batching replicates checks each one first and leaves the failing
 * ones out (calib/objective.py:47-70 runs each replicate in its own try). */
int lpg_check_desc(const lpg_sim_desc* sim);

/* Create a handle for n_sims simulations on CUDA device `device`.
 * Replaces SEIR_ABM.__init__ + the components setter as far as the device
 * state is concerned (model.py:101-175, 209-244). */
int lpg_create(const lpg_sim_desc* sims, int32_t n_sims, int32_t device, lpg_handle** out);

/* Bind the starting agent columns of simulation `sim` (copied; the caller
 * keeps ownership).  Replaces the implicit sharing of sim.people columns
 * between components (model.py:1288-1298). */
int lpg_bind_columns(lpg_handle* h, int32_t sim, const lpg_columns* cols);

/* Lay the bound columns out on the device and log tick 0
 * (SEIR_ABM.run at tick 0: log_results(0), model.py:253-256;
 * Transmission_ABM.log, model.py:1461-1487). */
int lpg_start(lpg_handle* h);

/* Advance every simulation by up to n_ticks ticks: for each tick the
 * components' step() in default_run_order then log(t)
 * (model.py:257-271; pars.py:99).  A simulation stops at nt or at its
 * early-stop tick.  Asynchronous: returns once the work is queued. */
int lpg_step(lpg_handle* h, int32_t n_ticks);

/* Wait for queued work; reports a sticky device-side error if one was set.
 * Device-side errors belong to one simulation (lpg_sim_state.error): a
 * simulation whose births exceed its capacity (LPG_ERR_CAPACITY), or whose
 * staged sweep gave up a bounded wait (LPG_ERR_TIMEOUT), stops at that tick
 * while the handle's other simulations run on.  lpg_sync returns the first
 * such error; read every simulation's own with lpg_get_state.  LPG_ERR_CUDA
 * is a failure of the whole handle. */
int lpg_sync(lpg_handle* h);

int lpg_get_state(lpg_handle* h, int32_t sim, lpg_sim_state* out);

/* Copy results of `sim` into caller arrays (sim.results.*). */
int lpg_read_results(lpg_handle* h, int32_t sim, const lpg_results_view* out);

/* Record, on every tick the transmission step runs, each node's inputs of
 * the expected-incidence map (lpg_incidence_plan_create) and the engine's own
 * expected new exposures; call before lpg_start.  No counterpart in the
 * reference.  The values are those of model.py:1315-1363 on that tick:
 * srisk = exposure_by_node (the susceptibles' summed acquisition risk),
 * beta = beta_by_node_strain before mixing, pop = results.pop[t], and
 * lam = expected_exposures_per_node. */
int lpg_record_aggregates(lpg_handle* h, int32_t sim, int32_t enable);
/* srisk, pop, lam [nt][n_nodes] and beta [nt][n_nodes][n_strains] (host;
 * any may be NULL).  Rows of ticks on which transmission did not run are 0. */
int lpg_read_aggregates(lpg_handle* h, int32_t sim, double* srisk, double* beta, double* pop, double* lam);

/* Copy the current agent columns of `sim` back in reference slot order
 * (slots [0, count) are written; slots past count are left untouched). */
int lpg_read_columns(lpg_handle* h, int32_t sim, const lpg_columns* out);

/* Diagnostic: recount every node total and selection weight from the agent
 * columns and compare with the running totals the engine maintains.
 * LPG_ERR_INTERNAL on any difference. */
int lpg_check_invariants(lpg_handle* h);

/* Use CUDA graphs for lpg_step (default on).  Off = plain launches. */
int lpg_set_graphs(lpg_handle* h, int32_t enable);

/* Per-kernel CUDA-event timing of lpg_step (forces plain launches).
 * Turning it on also sets the work counters below to zero. */
int lpg_set_profiling(lpg_handle* h, int32_t enable);
int lpg_read_profile(lpg_handle* h, lpg_profile* out);

/* Work counters the tick kernels accumulate on the device (all simulations
 * of the handle), from lpg_create or the last lpg_set_profiling(h, 1): the
 * data-dependent amounts of work behind each kernel's algorithmic bytes.
 * No counterpart in the reference. */
enum {
  LPG_CTR_SWEEP_INDEX = 0,   /* sub-block index entries k_due read */
  LPG_CTR_SWEEP_DUE = 1,     /* sub-blocks k_sweep_due visited (an event or a death due) */
  LPG_CTR_SWEEP_EVT_DUE = 2, /* of those, with an event due */
  LPG_CTR_SWEEP_DOD_DUE = 3, /* of those, with a death due */
  LPG_CTR_QUEUE_DS = 4,      /* queue entries of k_sweep_due (deaths, disease steps) */
  LPG_CTR_QUEUE_RS = 5,      /* queue entries of k_sweep_rs (RI, SIA) */
  LPG_CTR_SEL_TARGETS = 6,   /* targets k_select located, all rounds */
  LPG_CTR_SEL_NODE_ROUNDS = 7, /* node rounds after round 0 */
  LPG_CTR_RI_INDEX = 8,      /* RI due index entries k_sweep_rs read */
  LPG_CTR_RI_DUE = 9,        /* sub-blocks it visited with an RI due tick come */
  LPG_NUM_COUNTERS = 10
};
/* Copies min(n, LPG_NUM_COUNTERS) counters to out (host memory) after the
 * handle's stream has finished; returns LPG_OK or an error code. */
int lpg_read_counters(lpg_handle* h, uint64_t* out, int32_t n);

/* Test hook, no counterpart in the reference: the staged RI/SIA sweep's
 * producer issues at most `stages` stages per CTA (negative: all) and its
 * consumers give up a wait after `wait_spin` iterations (0: the normal
 * limit).  A withheld stage makes the consumers' bounded wait run out, as
 * a copy that never landed would: the CTA records LPG_ERR_TIMEOUT against
 * the simulations whose staged chunks it was sweeping, waits (on the normal
 * limit) for the copies it did issue, and returns.  Nothing faults and the
 * context stays usable.  Cached CUDA graphs are dropped. */
int lpg_test_stall_sweep(lpg_handle* h, int32_t stages, int64_t wait_spin);

/* Test hook of the same kind for the first selection round, whose CTAs meet
 * at a grid barrier (a cooperative launch: all of them resident): with
 * skip != 0, CTA 0 does not arrive, and the others give up their bounded
 * wait after `wait_spin` polls (0: the normal limit).  Every running
 * simulation then records LPG_ERR_TIMEOUT (the barrier's count is spent),
 * the kernel returns and the context stays usable.  Cached CUDA graphs are
 * dropped.  No counterpart in the reference. */
int lpg_test_stall_round0(lpg_handle* h, int32_t skip, int64_t wait_spin);

/* Grid sizes (CTAs) of the tick kernels, after lpg_start: the engine's
 * default is every CTA that fits at once (occupancy x SM count, capped);
 * an autotuner may set others.  Results do not depend on them (every kernel
 * is a grid-stride or work-split loop over exact integer updates), only the
 * time does.  Setting one drops the cached CUDA graphs.  No counterpart in
 * the reference.  lpg_set_launch returns LPG_ERR_ARG outside [1, the
 * kernel's limit] (1024 for the two sweeps, whose per-CTA queue slabs are
 * sized for that, and for k_sel_rounds; for k_sel_round0, a cooperative
 * launch, the CTAs that fit on the GPU at once; 8192 for the others);
 * lpg_get_launch returns the size, or a negative lpg_status. */
enum {
  LPG_LAUNCH_DUE = 0,       /* k_due */
  LPG_LAUNCH_SWEEP_DUE = 1, /* k_sweep_due */
  LPG_LAUNCH_SWEEP_RS = 2,  /* k_sweep_rs (and the slabs k_evb reads) */
  LPG_LAUNCH_EVB = 3,       /* k_evb */
  LPG_LAUNCH_SELECT = 4,    /* k_sel_round0 (cooperative: at most the CTAs resident at once) */
  LPG_LAUNCH_ROUNDS = 5,    /* k_sel_rounds */
  LPG_LAUNCH_NEWBORNS = 6,  /* k_newborns (CTAs per replicate) */
  LPG_NUM_LAUNCH = 7
};
int lpg_set_launch(lpg_handle* h, int32_t which, int32_t blocks);
int lpg_get_launch(lpg_handle* h, int32_t which);

/* The CUDA stream the handle launches on, as an opaque pointer. */
void* lpg_cuda_stream(lpg_handle* h);

/* Number of kernel launches the handle has issued (graph replays count
 * every kernel node). */
int64_t lpg_kernel_launches(lpg_handle* h);

const char* lpg_last_error(const lpg_handle* h);
void lpg_destroy(lpg_handle* h);

/* ---------------------------------------------------------------------- */
/* Initialisation of the agent table on the device.
 *
 * The reference fills its columns in SEIR_ABM.__init__ and in each
 * component's constructor with numpy draws (model.py:101-175, 561-713,
 * 816-866, 1548-1611, 1887-1894; flagged slow at :852).  lpg_init_columns
 * fills the same columns with this project's counter-based draws, in
 * reference slot order, on the device.  `parts` selects what to fill, in the
 * order of the bits below; a part reads what earlier parts (of this call or
 * an earlier one) wrote.  Each part writes the columns named beside it, over
 * the whole capacity:
 *   LPG_INIT_BASE        disease_state (0 for the first count slots, -1 after),
 *                        node_id (node-contiguous from node_pop, -1 after),
 *                        strain 0, potentially_paralyzed -1, paralyzed 0,
 *                        ipv_protected 0, chronically_missed 0 (model.py:139-162)
 *   LPG_INIT_MISSED      chronically_missed = 1 for missed_k agents chosen
 *                        without replacement among the first count (:155-158)
 *   LPG_INIT_TIMERS      exposure_timer, infection_timer, paralysis_timer (:575-587)
 *   LPG_INIT_IMMUNITY    disease_state = 3 for immune_k[n] agents of each node,
 *                        chosen without replacement (:589-618)
 *   LPG_INIT_PREVALENCE  disease_state = 2 for prev_k agents chosen among all
 *                        (prev_per_node 0, prev_k[0]) or prev_k[n] per node (:670-713)
 *   LPG_INIT_HETEROGENEITY acq_risk_multiplier, daily_infectivity (:816-866)
 *   LPG_INIT_AGES        date_of_birth (-age for the first count, -1 after) (:1576-1596)
 *   LPG_INIT_DEATHS      date_of_death (age at death - age; 0 after) (:1605-1611)
 *   LPG_INIT_RI          ri_timer (date of birth + [42, 98) days; -1 after) (:1887-1894)
 * Selections take the agents with the smallest counter-based keys (exactly
 * k of the group, every subset equally likely).  Column pointers are device
 * memory of `capacity` elements; only those a requested part writes or reads
 * need be set.  Asynchronous on `stream`; scratch comes from
 * cudaMallocAsync on it.  Errors: lpg_op_last_error(). */
enum {
  LPG_INIT_BASE = 1,
  LPG_INIT_MISSED = 2,
  LPG_INIT_TIMERS = 4,
  LPG_INIT_IMMUNITY = 8,
  LPG_INIT_PREVALENCE = 16,
  LPG_INIT_HETEROGENEITY = 32,
  LPG_INIT_AGES = 64,
  LPG_INIT_DEATHS = 128,
  LPG_INIT_RI = 256
};

typedef struct {
  int32_t n_nodes;
  int32_t prev_per_node;     /* LPG_INIT_PREVALENCE: 1 = prev_k[n] per node, 0 = prev_k[0] among all */
  int64_t count, capacity;
  uint64_t seed;
  const int64_t* node_pop;   /* [n_nodes] initial agents per node (pars.init_pop) */
  int64_t missed_k;          /* int(missed_frac * count) */
  const int64_t* immune_k;   /* [n_nodes] int(immunity fraction * node pop) */
  const int64_t* prev_k;     /* [n_nodes] or [1] */
  lpg_dist dur_exp, dur_inf, t_to_paralysis;
  int32_t heterogeneity;     /* pars.individual_heterogeneity */
  int32_t n_age_bins;
  double risk_mult_var, corr_risk_inf;
  double r0;                 /* infectivity mean = r0 / mean of 1000 infectious durations */
  const int32_t* age_lo_days;  /* [n_age_bins] inclusive: max(min age * 365, 1) */
  const int32_t* age_hi_days;  /* [n_age_bins] exclusive: (max age + 1) * 365 */
  const int64_t* age_weight;   /* [n_age_bins] */
  const int64_t* km_cumdeaths; /* cumulative deaths by age-year (utils.py:795-816) */
  int32_t km_len, km_max_year;
} lpg_init_desc;

int lpg_init_columns(const lpg_init_desc* d, uint32_t parts, const lpg_columns* cols, void* stream);

/* The mean daily infectivity the initialisation scales to,
 * r0 / mean(dur_inf(1000)) (model.py:843; the mean of 1000 draws, as the
 * reference estimates it), with this project's draws.  Host only. */
double lpg_init_mean_infectivity(uint64_t seed, double r0, lpg_dist dur_inf);

/* ---------------------------------------------------------------------- */
/* Standalone ops over plain device columns (no handle).  Asynchronous on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) on the
 * current device.  Errors: a negative lpg_status; the text from
 * lpg_op_last_error() (per host thread). */

#define LPG_COUNT_SEIRP_MAX_NODES 4096

/* count_SEIRP (laser_polio/model.py:869-899, kernel :902-929): per-node
 * counts of slots [0, n_people) with disease_state >= 0 — S, E, I, R
 * [n_nodes]; E_by_strain, I_by_strain [n_nodes][n_strains];
 * potentially_paralyzed == 1 as POTP, paralyzed == 1 as P [n_nodes].
 * Columns and outputs are device pointers; outputs are overwritten.  Slots
 * with a node id outside [0, n_nodes), or E/I slots with a strain outside
 * [0, n_strains), are not counted; their number goes to *n_invalid (device
 * int64, may be NULL).  Scratch: cudaMallocAsync on `stream`. */
int lpg_count_seirp(const int16_t* node_id, const int8_t* disease_state, const int8_t* strain,
                    const int8_t* potentially_paralyzed, const int8_t* paralyzed, int32_t n_nodes, int32_t n_strains,
                    int64_t n_people, int32_t* S, int32_t* E, int32_t* I, int32_t* R, int32_t* E_by_strain,
                    int32_t* I_by_strain, int32_t* POTP, int32_t* P, int64_t* n_invalid, void* stream);

/* lpg_count_seirp without any device allocation, for callers that cannot
 * allocate device memory at call time (a process whose device memory is
 * claimed by its own caching pool; a loop that must not stall the device,
 * which cudaFree does).  No counterpart in the reference (its count_SEIRP
 * allocates numpy tables on every call).  Same arguments and results as
 * lpg_count_seirp; n_nodes is limited the same way (LPG_COUNT_SEIRP_MAX_NODES),
 * and a histogram larger than the static scratch is rejected with
 * LPG_ERR_ARG.
 *   - Scratch: a file-scope device array of LPG_COUNT_SEIRP_STATIC_WORDS
 *     int32 words (4 MiB) per device; nothing in it needs to start at zero.
 *   - The first call on each device looks up the array's device address with
 *     that device current; make that first call before any stream capture.
 *   - All calls on a device share the array: calls whose kernels overlap on
 *     the GPU race and may return wrong counts.  Serialize them (one stream). */
#define LPG_COUNT_SEIRP_STATIC_WORDS (1 << 20)
int lpg_count_seirp_static(const int16_t* node_id, const int8_t* disease_state, const int8_t* strain,
                           const int8_t* potentially_paralyzed, const int8_t* paralyzed, int32_t n_nodes,
                           int32_t n_strains, int64_t n_people, int32_t* S, int32_t* E, int32_t* I, int32_t* R,
                           int32_t* E_by_strain, int32_t* I_by_strain, int32_t* POTP, int32_t* P,
                           int64_t* n_invalid, void* stream);

/* Expected incidence of a replayed tick range and its vector-Jacobian
 * product, for gradient-based calibration.  No counterpart in the reference
 * (its calibration samples parameters with Optuna, laser_polio/calibration,
 * and differentiates nothing).  With the agent state held fixed, the
 * node-level part of the transmission step (model.py:1315-1363) maps
 * per-tick aggregates to the expected new exposures
 *   N        = rownorm(gravity(pops, dist, k, a, b, c) / (sum pops)^c, max_frac)
 *                                                   (model.py:1250-1258)
 *   u[t,n,s] = beta[t,n,s] (1 - sum_j N[n,j]) + sum_i N[i,n] beta[t,i,s]
 *   seas[t]  = 1 + amp cos(2 pi (doy[t] - peak) / year[t])  (utils.py:589-625)
 *   lam[t,n] = srisk[t,n] sum_s (1 - exp(-u seas[t] r0s[n] R / max(pop[t,n], 1)))
 * gravity[i][j] = k pops_i^a pops_j^b / dist_ij^c off the diagonal, 0 on it;
 * a row whose sum exceeds max_frac is scaled down to max_frac.  R scales
 * every agent's infectivity (R0 over the R0 the aggregates were taken at).
 * All arrays are host, row-major FP64. */
typedef struct {
  int32_t T, G, S;    /* ticks, nodes, strains (S <= LPG_MAX_STRAINS) */
  const double* srisk; /* [T][G] susceptibles' summed acquisition risk */
  const double* beta;  /* [T][G][S] summed infectivity before mixing */
  const double* pop;   /* [T][G] node population */
  const double* doy;   /* [T] day of year of each tick */
  const double* year;  /* [T] days in that year */
  const double* r0s;   /* [G] per-node R0 scalars */
  const double* pops;  /* [G] gravity populations */
  const double* dist;  /* [G][G] distances (the diagonal is ignored) */
  double R, amp, peak; /* infectivity scale, seasonal amplitude, peak day */
  double k, a, b, c;   /* gravity parameters */
  double max_frac;     /* row-sum cap of the network */
} lpg_incidence_in;

typedef struct {
  double R, amp, peak, k, a, b, c; /* dL/d of each scalar */
  double* r0s;                     /* [G] dL/dr0s, or NULL */
  double* network;                 /* [G][G] dL/dN (zero diagonal), or NULL */
} lpg_incidence_grad;

/* The parameters a calibration varies, per evaluation. */
typedef struct {
  double R, amp, peak, k, a, b, c, max_frac;
  const double* r0s; /* [G] host */
} lpg_incidence_params;

/* A plan keeps the aggregates (and an optional target curve) resident on
 * the current device and evaluates the map at any parameters without
 * re-uploading them.  Not thread-safe; calls on one plan are serialized. */
typedef struct lpg_incidence_plan lpg_incidence_plan;

/* Copies in's arrays (r0s and the scalars are not used) and, if non-NULL,
 * target [T][G] (host) to the device.  stream: a cudaStream_t the plan
 * works on, or NULL for a stream of its own. */
int lpg_incidence_plan_create(const lpg_incidence_in* in, const double* target, void* stream,
                              lpg_incidence_plan** out);

/* One evaluation at *prm, synchronous:
 *   lam_out  [T][G] host, or NULL: lam;
 *   loss_out (needs a target), or NULL: L = sum (log1p(lam) - log1p(target))^2;
 *   grad     or NULL: the gradients of L = sum g_lam * lam when g_lam
 *            ([T][G] host) is given, else of the target loss. */
int lpg_incidence_plan_eval(lpg_incidence_plan* p, const lpg_incidence_params* prm, const double* g_lam,
                            double* lam_out, double* loss_out, lpg_incidence_grad* grad);
void* lpg_incidence_plan_stream(lpg_incidence_plan* p);
/* Per-kernel device time (CUDA events on the plan's stream) of the
 * evaluations made while profiling is on; enabling resets the sums. */
int lpg_incidence_plan_set_profiling(lpg_incidence_plan* p, int32_t enable);
int lpg_incidence_plan_read_profile(lpg_incidence_plan* p, lpg_profile* out);
void lpg_incidence_plan_destroy(lpg_incidence_plan* p);

/* One-shot: a plan on `stream`, one evaluation at in's parameters, freed.
 * lam_out [T][G] (host) receives lam.  With g_lam non-NULL ([T][G], host:
 * dL/dlam), *grad receives the gradients of L = sum g_lam * lam.
 * Reductions use atomics: results match a sequential FP64 evaluation to
 * rounding, not bit for bit.  Errors: lpg_op_last_error(). */
int lpg_expected_incidence(const lpg_incidence_in* in, double* lam_out, const double* g_lam,
                           lpg_incidence_grad* grad, void* stream);

/* save_sim_results' table (utils.py:689-786) as CSV, written by host threads:
 * one row per (timestep, node), timestep-major, with the columns timestep,
 * date, node, dot_name, then field_names[0..n_fields), then the summary
 * groupings' string columns (utils.py:1040-1160): n_tick_cols by tick
 * (tick_cols[c * nt + t], e.g. time_period) and then n_node_cols by node
 * (node_cols[c * n_nodes + n], e.g. adm0, adm1, adm01, region).  The format
 * of pandas' DataFrame.to_csv(index=False) ('\n' rows, QUOTE_MINIMAL
 * strings).  dates [nt] and dot_names [n_nodes] are NUL-terminated strings;
 * fields[k] is an int32 array [nt][n_nodes].  Host memory only; needs no GPU. */
#define LPG_EXPORT_MAX_FIELDS 64
int lpg_write_results_csv(const char* path, int32_t nt, int32_t n_nodes, const char* const* dates,
                          const char* const* dot_names, int32_t n_fields, const char* const* field_names,
                          const int32_t* const* fields, int32_t n_tick_cols, const char* const* tick_col_names,
                          const char* const* tick_cols, int32_t n_node_cols, const char* const* node_col_names,
                          const char* const* node_cols);

/* The radiation migration network (the reference builds it with laser_core's
 * radiation at model.py:1252-1254; migration_method's default): out[i][j] =
 * k p_i p_j / ((p_i + s_ij)(p_i + p_j + s_ij)), s_ij the population of the
 * nodes other than i and j strictly closer to i than j (nodes tied with j
 * are outside), zero diagonal.  include_home must be 0 (the reference only
 * builds include_home=False): LPG_ERR_ARG otherwise.  Host arrays, row-major
 * [n][n]; rows on host threads; no GPU.  Equal bit for bit to
 * laser_polio_gb300.core's Python definition. */
int lpg_radiation_network(const double* pops, const double* dist, int32_t n, double k, int32_t include_home,
                          double* out);

const char* lpg_op_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* LPG_H */
