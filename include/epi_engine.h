/*
 * epi_engine.h -- C ABI of the GB300 engine tick for EpiRust-style agent simulations.
 *
 * One engine handle owns one single-region simulation (one "engine" in EpiRust terms):
 * the agents live on the GPU as struct-of-arrays state over a dense occupancy plane, and
 * the host keeps the configuration, the hourly run loop, the intervention triggers and the
 * counts/CSV output.  Every function returns an int status (EPI_OK == 0) and never aborts.
 *
 * Each entry point names the reference interface it replaces (paths are relative to the
 * thoughtworks/epirust source tree).
 */
#ifndef EPI_ENGINE_H
#define EPI_ENGINE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
/* The reference panics/asserts (engine/src/allocation_map.rs:128, 175-179;
 * engine/src/epidemiology_simulation.rs:228-230); here every failure is a status code. */
enum {
    EPI_OK = 0,
    EPI_ERR_CONFIG = 1,    /* invalid or unsupported configuration                       */
    EPI_ERR_CAPACITY = 2,  /* population does not fit (houses full, too many infections) */
    EPI_ERR_CUDA = 3,      /* a CUDA runtime call failed                                  */
    EPI_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up                          */
    EPI_ERR_INVARIANT = 5, /* a consistency check failed (counts total != population)    */
    EPI_ERR_ARG = 6,       /* bad argument (null pointer, short buffer, hour out of range) */
    EPI_ERR_IO = 7         /* a file could not be written, read or was not what it claims   */
};

/* ---------------------------------------------------------------- enumerations */
/* Disease state, flattening engine/src/state_machine/state.rs:22-37
 * (State x Severity) into one code. */
enum {
    EPI_S = 0,          /* Susceptible                         */
    EPI_E = 1,          /* Exposed { at_hour }                 */
    EPI_I_PRE = 2,      /* Infected { day, Pre { at_hour } }   */
    EPI_I_ASYM = 3,     /* Infected { day, Asymptomatic }      */
    EPI_I_MILD = 4,     /* Infected { day, Mild }              */
    EPI_I_SEVERE = 5,   /* Infected { day, Severe }            */
    EPI_R = 6,          /* Recovered                           */
    EPI_D = 7           /* Deceased                            */
};

/* engine/src/citizen/work_status.rs:23-28 */
enum { EPI_WS_NORMAL = 0, EPI_WS_ESSENTIAL = 1, EPI_WS_HOSPITAL_STAFF = 2, EPI_WS_NA = 3 };

/* epi_agent_record.flags bits (engine/src/citizen/mod.rs:48-63) */
enum {
    EPI_F_HOSPITALIZED = 1,
    EPI_F_ISOLATED = 2,
    EPI_F_VACCINATED = 4,
    EPI_F_WORK_QUARANTINED = 8,
    EPI_F_PUBLIC_TRANSPORT = 16
};

/* Intervention bits reported by epi_engine_process_interventions. */
enum {
    EPI_IV_VACCINATION = 1,
    EPI_IV_LOCKDOWN = 2,
    EPI_IV_LOCKDOWN_REVOKED = 4,
    EPI_IV_BUILD_NEW_HOSPITAL = 8
};

#define EPI_MAX_VACCINATIONS 32

/* ---------------------------------------------------------------- records */
/* One CSV row; field order of engine/src/models/events/counts.rs:25-34. */
typedef struct {
    uint32_t hour, susceptible, exposed, infected, hospitalized, recovered, deceased;
} epi_counts;

/* Flat form of the simulation config JSON (common/src/config/mod.rs:44-58).  Only the
 * Auto population and an inline disease are supported by the standalone engine. */
typedef struct {
    /* population: Auto (common/src/config/population.rs:36-43) */
    uint32_t number_of_agents;
    double public_transport_percentage;
    double working_percentage;
    /* geography_parameters (common/src/config/geography_parameters.rs:23-28) */
    uint32_t grid_size;
    double hospital_beds_percentage;
    /* hours of the run loop: simulated hours are 1 .. hours-1 */
    uint32_t hours;
    /* disease (common/src/disease/mod.rs:26-45) */
    uint32_t regular_transmission_start_day;
    uint32_t high_transmission_start_day;
    uint32_t last_day;
    uint32_t asymptomatic_last_day;  /* parsed, unused: the engine uses the constant 9  */
    uint32_t mild_infected_last_day; /* parsed, unused: the engine uses the constant 12 */
    double regular_transmission_rate;
    double high_transmission_rate;
    double death_rate;
    double percentage_asymptomatic_population;
    double percentage_severe_infected_population;
    uint32_t exposed_duration;
    uint32_t pre_symptomatic_duration;
    /* starting_infections (common/src/config/starting_infections.rs:22-69) */
    uint32_t infected_mild_asymptomatic;
    uint32_t infected_mild_symptomatic;
    uint32_t infected_severe;
    uint32_t exposed;
    /* interventions (common/src/config/intervention_config.rs:23-48); the first Lockdown
     * and the first BuildNewHospital entry are used, Vaccinate entries are keyed by hour */
    int32_t has_lockdown;
    uint32_t lockdown_at_number_of_infections;
    double essential_workers_population;
    int32_t has_build_new_hospital;
    uint32_t spread_rate_threshold;
    int32_t n_vaccinations;
    uint32_t vaccination_at_hour[EPI_MAX_VACCINATIONS];
    double vaccination_percent[EPI_MAX_VACCINATIONS];
    /* extension (no reference counterpart): build the new hospital at a day boundary when
     * hospitalized >= fraction x hospital cells; <= 0 disables it */
    double hospital_occupancy_trigger;
    /* extension: counter-based random stream key (the reference RNG is unseeded) */
    uint64_t seed;
    /* Population source: 0 Auto (number_of_agents and the two percentages), 1 Csv (one row
     * per agent, common/src/config/population.rs:31-34; the rows come with
     * epi_engine_create_population and number_of_agents is their count). */
    uint32_t population_source;
    char population_file[256];  /* Csv: the "file" of the config (NUL-terminated) */
} epi_params;

/* Per-agent snapshot (host layout, used for oracle comparison and checkpoints).
 * at_hour is meaningful for EPI_E and EPI_I_PRE, infection_day for EPI_I_*,
 * work_start_at for hospital staff; all are 0 otherwise. */
typedef struct {
    int32_t x, y;
    uint8_t state, flags, work_status;
    int8_t immunity;
    uint32_t at_hour;
    uint32_t infection_day;
    uint32_t work_start_at;
    int32_t home_x, home_y;  /* start corner of the 2x2 house   */
    int32_t work_x, work_y;  /* start corner of the 10x10 office */
    int32_t area_x0, area_y0, area_x1, area_y1; /* current_area rectangle (inclusive) */
} epi_agent_record;

/* Area rectangle (inclusive corners), engine/src/geography/area.rs:30-35. */
typedef struct { int32_t x0, y0, x1, y1; } epi_area;

/* Grid layout, engine/src/geography/grid.rs:36-50 (houses/offices as counts + origin). */
typedef struct {
    uint32_t grid_size;
    epi_area housing, transport, work, hospital;
    uint32_t houses_x, houses_y;   /* area_factory(housing, 2) tiling  */
    uint32_t offices_x, offices_y; /* area_factory(work, 10) tiling    */
} epi_geography;

typedef struct epi_engine epi_engine;

/* ---------------------------------------------------------------- config + geography */
/* Config::read (common/src/config/mod.rs:119-123): parse the engine's JSON config.
 * Unknown keys are ignored, like serde's default.  err (may be NULL) gets a message. */
int epi_params_from_json(const char* json, epi_params* out, char* err, size_t errlen);

/* geography::define_geography (engine/src/geography/mod.rs:33-70). */
int epi_define_geography(uint32_t grid_size, epi_geography* out);

/* Grid::resize_hospital (engine/src/geography/grid.rs:240-261), applied to geo->hospital. */
int epi_resize_hospital(epi_geography* geo, int32_t number_of_agents,
                        double hospital_staff_percentage, double hospital_beds_percentage);

/* Grid::increase_hospital_size (engine/src/geography/grid.rs:233-238): the hospital keeps
 * its start corner and ends at (grid_size, grid_size). */
int epi_geography_increase_hospital_size(epi_geography* geo, uint32_t grid_size);

/* The trigger logic of process_interventions (allocation_map.rs:306-337 with
 * interventions/{vaccination,lockdown,hospital}.rs) on the host alone, for checks without a
 * device: from a fresh intervention state the rows are offered in order, as the run loop
 * offers every hour's counts.  applied[k] gets the EPI_IV_* bits that fire at rows[k].
 * guard[k] (may be NULL) gets 1 where the run loop's device guard would mark rows[k] to halt
 * its chain: a day boundary at which a lockdown or a hospital build is due, judged from the
 * thresholds in force before that row. */
int epi_interventions_replay(const epi_params* params, const epi_counts* rows, uint32_t n, uint32_t* applied,
                             uint8_t* guard);

/* The listeners' files for a run's rows, without a device: CsvListener's
 * <dir>/output/simulation_<engine_id>_<UTC YYYY-MM-DDTHH:MM:SS>.csv (header hour, susceptible,
 * exposed, infected, hospitalized, recovered, deceased; one line per row) and
 * InterventionReporter's ..._interventions.json, whose reports come from replaying the
 * intervention triggers over the rows (util.rs:36-43, csv_service.rs:44-71,
 * intervention_reporter.rs:52-58).  epi_engine_write_outputs writes the same files from an
 * engine's own run. */
int epi_outputs_write(const char* dir, const char* engine_id, const epi_params* params, const epi_counts* rows,
                      uint32_t n);

/* Disease::get_current_transmission_rate / is_to_be_hospitalized
 * (common/src/disease/mod.rs:88-99). */
double epi_disease_transmission_rate(const epi_params* p, uint32_t infection_day);
int epi_disease_is_to_be_hospitalized(const epi_params* p, uint32_t infection_day);

/* Csv population (grid.rs:194-231, citizen/population_record.rs): read the columns
 * "working" and "pub_transport" ("True" / "False") of every row into flags (bit 0 working,
 * bit 1 public transport).  flags may be NULL to count the rows; at most cap are written. */
int epi_population_read_csv(const char* path, uint8_t* flags, uint32_t cap, uint32_t* n);
/* World build / engine from per-agent population flags (n == params->number_of_agents):
 * agent i gets house i mod houses and office i mod offices (the cycled iterators of
 * read_population), working and public transport from its flags, and the rest as in the
 * Auto build (Citizen::from_record, citizen/mod.rs:155-180). */
int epi_world_build_population(const epi_params* params, const uint8_t* flags, uint32_t n, epi_agent_record* out,
                               epi_geography* geo);
int epi_engine_create_population(const epi_params* params, const uint8_t* flags, uint32_t n, epi_engine** out);

/* World build of Epidemiology::new (engine/src/epidemiology_simulation.rs:85-117):
 * geography, Auto population, starting infections, hospital resize and essential
 * workers, on the host.  Fills n records (n must equal number_of_agents). */
int epi_world_build(const epi_params* p, epi_agent_record* out, size_t n, epi_geography* geo);

/* ---------------------------------------------------------------- engine */
/* Epidemiology::new (engine/src/epidemiology_simulation.rs:75-135): builds the world and
 * uploads it to cuda device 0 (or the current device). */
int epi_engine_create(const epi_params* params, epi_engine** out);

/* Same, from the JSON config text; seed overrides the config's optional "seed" key. */
int epi_engine_create_json(const char* config_json, uint64_t seed, epi_engine** out);

/* Same, from host-side records (a world built elsewhere or a checkpoint).  The records are
 * copied to the device as they are (pinned host memory makes that one DMA) and checked and
 * packed there: a cell, house, office or current area outside [0, grid_size], a state, work
 * status, immunity or infection day beyond its field, or a current area that is none of the
 * agent's areas returns EPI_ERR_ARG, and epi_engine_last_error(NULL) names the first such
 * record. */
int epi_engine_create_from_records(const epi_params* params, const epi_agent_record* recs,
                                   size_t n, epi_engine** out);

void epi_engine_destroy(epi_engine* h);

/* Message of the last failure on this handle (or of the last failed create on this
 * thread when h is NULL). */
const char* epi_engine_last_error(const epi_engine* h);

/* Run the engine's work on this cudaStream_t (NULL = the engine's own stream). */
int epi_engine_set_stream(epi_engine* h, void* cuda_stream);

/* CitizenLocationMap::simulate (engine/src/allocation_map.rs:67-129): one hour
 * (move, infect, count); counts->hour is set to hour. */
int epi_engine_simulate(epi_engine* h, uint32_t hour, epi_counts* out);

/* n consecutive hours first_hour .. first_hour+n-1 with no interventions in between,
 * issued as captured CUDA graphs of whole days launched back to back; out gets n rows. */
int epi_engine_simulate_hours(epi_engine* h, uint32_t first_hour, uint32_t n, epi_counts* out);

/* CitizenLocationMap::process_interventions (engine/src/allocation_map.rs:306-337) with
 * the trigger logic of engine/src/interventions/{vaccination,lockdown,hospital}.rs.
 * counts are this hour's counts; *applied gets EPI_IV_* bits (may be NULL). */
int epi_engine_process_interventions(epi_engine* h, const epi_counts* counts, uint32_t* applied);

/* The bulk agent updates behind the interventions. */
int epi_engine_lock_city(epi_engine* h);                        /* allocation_map.rs:349-356 */
int epi_engine_unlock_city(epi_engine* h);                      /* allocation_map.rs:358-365 */
int epi_engine_vaccinate(epi_engine* h, uint32_t hour, double percent); /* allocation_map.rs:381-387 */
int epi_engine_increase_hospital_size(epi_engine* h);           /* grid.rs:233-238 */

/* Epidemiology::run_single_engine (engine/src/epidemiology_simulation.rs:211-274):
 * hours 1 .. hours-1 with interventions and the standalone stop rule.  rows gets one
 * epi_counts per simulated hour (capacity max_rows >= hours-1); *n_rows the number written.
 * A run paused by epi_engine_run_until continues where it stopped (rows from hour 1). */
int epi_engine_run(epi_engine* h, epi_counts* rows, uint32_t max_rows, uint32_t* n_rows);

/* The same run loop, paused after hour last_hour (no reference counterpart): rows so far as
 * epi_engine_run gives them; *next_hour is the hour the run continues from, or 0 when it has
 * ended.  Direct hour calls (epi_engine_simulate*) do not advance a paused run. */
int epi_engine_run_until(epi_engine* h, uint32_t last_hour, epi_counts* rows, uint32_t max_rows, uint32_t* n_rows,
                         uint32_t* next_hour);

/* On-disk checkpoint of a single engine (no reference counterpart): the parameters, the
 * current geography, every agent record, the intervention state and reports, the rows and
 * the position of a paused run.  With counter-based random streams the resumed run is the
 * uninterrupted one, bit for bit.  File: "EPCK", version, struct sizes, then the parts in
 * that order and an FNV-1a 64 checksum of everything before it.  A file that is missing,
 * truncated, of another version or whose checksum differs gives EPI_ERR_IO. */
int epi_engine_checkpoint_write(epi_engine* h, const char* path);
int epi_engine_create_from_checkpoint(const char* path, epi_engine** out);

/* Listeners: CsvListener + InterventionReporter (engine/src/listeners/csv_service.rs:61-71,
 * intervention_reporter.rs:52-63).  Writes <dir>/output/simulation_<engine_id>_<UTC time>.csv
 * and <same>_interventions.json for the rows of the last epi_engine_run
 * (engine/src/utils/util.rs:28-43). */
int epi_engine_write_outputs(epi_engine* h, const char* dir, const char* engine_id);

/* CitizenLocationMap::current_population (engine/src/allocation_map.rs:389-391). */
int epi_engine_population(const epi_engine* h, uint32_t* out);

/* Copy all agents back to the host (n == population). */
int epi_engine_snapshot(epi_engine* h, epi_agent_record* out, size_t n);

/* Current geography (the hospital changes after BuildNewHospital). */
int epi_engine_geography(const epi_engine* h, epi_geography* out);

/* Check the device invariants: every agent sits on its own plane cell and the plane holds
 * exactly population occupied cells. */
int epi_engine_check(epi_engine* h);

/* Device-side checkpoint of the agent state, the plane, the intervention state, the
 * hospital and the position of a paused run (the reference has none; its counts live only in
 * memory until the end, engine/src/listeners/csv_service.rs:61-71).  restore_state rewinds
 * to the last save; with counter-based random streams a rewound run repeats itself exactly. */
int epi_engine_save_state(epi_engine* h);
int epi_engine_restore_state(epi_engine* h);

/* Number of engine kernels launched so far on this handle (graph nodes included). */
int epi_engine_kernels_launched(const epi_engine* h, uint64_t* out);

/* Launch shape of the tick kernels: the k_decide / k_sleep grid and the agents per k_commit
 * thread (its grid covers every agent once).  Results never depend on it. */
typedef struct {
    uint32_t decide_blocks;  /* 1 .. number of 256-agent chunks */
    uint32_t commit_slots;   /* 1 .. 8 */
    double hour_us;          /* autotune: mean wall time of a simulated hour with this shape */
} epi_launch_shape;

/* Citizen-state stream: the reference's CitizenStatesAtHr messages (every agent's state
 * letter s/e/i/r/d and cell, every hour; models/events/citizen_state.rs:27-70, published from
 * allocation_map.rs:122-124 when enable_citizen_state_messages is set) written to a file.
 * After a keyframe (every agent's cell and letter), each simulated hour is encoded on the
 * device as one byte per agent -- the Moore step taken (0 none, 1..8 in NeighborIterator
 * order, 15 a jump listed separately with its cell) and the state letter -- and appended as
 * {hour, agents, jumps} (u32), the bytes, then the jumps {agent, x | y << 16} in agent order.
 * epirust_gb300/state_stream.py reads the file back.  Single engines only. */
int epi_engine_state_stream_open(epi_engine* h, const char* path);
int epi_engine_state_stream_close(epi_engine* h);

/* Autotuner (no reference counterpart): time hours 1..hours (<= 168) of the current world
 * under each candidate shape -- k_decide grid = three quarters of the resident blocks, the
 * resident blocks, twice that, or one chunk per block; 1, 2 or 4 agents per k_commit thread --
 * from the same starting state, keep the fastest and restore the state.  Call it before simulating; it replaces the checkpoint of
 * epi_engine_save_state. */
int epi_engine_autotune(epi_engine* h, uint32_t hours, epi_launch_shape* chosen);
int epi_engine_set_launch_shape(epi_engine* h, const epi_launch_shape* shape);
int epi_engine_launch_shape(const epi_engine* h, epi_launch_shape* out);

/* Kernel timing: when enabled, every kernel launch of the engine is bracketed by CUDA
 * events on the launching stream and CUDA graphs are not used.  kernel_stats returns, per
 * kernel kind k < n, its launch count and total milliseconds; names via kernel_name. */
int epi_engine_set_profiling(epi_engine* h, int on);
int epi_engine_kernel_stats(const epi_engine* h, uint32_t* launches, double* total_ms, int n);
const char* epi_engine_kernel_name(int k);
int epi_engine_kernel_kinds(void);

/* sizeof of a public struct by name ("epi_params", "epi_agent_record", "epi_counts",
 * "epi_geography"), so an FFI binding can check its layout; 0 for unknown names. */
size_t epi_abi_struct_size(const char* name);

/* Algorithmic bytes of one hour at the current state (the roofline numerator). */
int epi_engine_hour_bytes(const epi_engine* h, uint32_t hour, double* bytes);

/* ---------------------------------------------------------------- batched ensemble */
/* No counterpart in the reference (it runs one world per process; many runs mean many
 * processes).  R independent worlds -- each with its own population, grid, disease, seed,
 * hours and interventions -- share one device and advance together: every kernel of an hour
 * serves all of them in one launch, hour segments are replayed as CUDA graphs.  Replicate r
 * evolves exactly as a single engine created from params[r] would. */
typedef struct epi_ensemble epi_ensemble;

int epi_ensemble_create(const epi_params* params, uint32_t replicates, epi_ensemble** out);
void epi_ensemble_destroy(epi_ensemble* e);
const char* epi_ensemble_last_error(const epi_ensemble* e);
int epi_ensemble_set_stream(epi_ensemble* e, void* cuda_stream);
int epi_ensemble_replicates(const epi_ensemble* e, uint32_t* out);

/* run_single_engine for every replicate (each with its own hours, interventions and stop
 * rule).  rows[r * max_rows_per_replicate + k] gets hour k+1 of replicate r; n_rows[r] the
 * number of rows of replicate r. */
int epi_ensemble_run(epi_ensemble* e, epi_counts* rows, uint32_t max_rows_per_replicate, uint32_t* n_rows);

int epi_ensemble_snapshot(epi_ensemble* e, uint32_t replicate, epi_agent_record* out, size_t n);
int epi_ensemble_check(epi_ensemble* e);
int epi_ensemble_save_state(epi_ensemble* e);
int epi_ensemble_restore_state(epi_ensemble* e);
int epi_ensemble_set_profiling(epi_ensemble* e, int on);
int epi_ensemble_kernel_stats(const epi_ensemble* e, uint32_t* launches, double* total_ms, int n);
int epi_ensemble_kernels_launched(const epi_ensemble* e, uint64_t* out);
/* epi_engine_autotune for all replicates together. */
int epi_ensemble_autotune(epi_ensemble* e, uint32_t hours, epi_launch_shape* chosen);
int epi_ensemble_hour_bytes(const epi_ensemble* e, uint32_t hour, double* bytes);

/* ---------------------------------------------------------------- no-allocation hour */
/* No counterpart in the reference.  One simulated hour (the work of epi_engine_simulate) on
 * device arrays that the caller owns, for callers that cannot allocate device memory: a host
 * runtime whose device memory comes from its own fixed pool or arena and may not grow behind
 * its back, or a real-time loop that must not enter the driver's allocator (cudaMalloc can
 * block on a device-wide synchronisation and take milliseconds).  This entry
 * point calls no cudaMalloc, cudaFree or allocating library routine; its scratch (parameter
 * block, per-agent proposal buffer, (G+1)^2 claim plane) is one fixed 48 MiB device array
 * inside the library, which every GPU that loads the library holds until the process exits.
 * A world needs 512 + 4 N bytes of it, rounded up to a multiple of 256, plus 4 (G+1)^2 bytes;
 * a larger one is rejected with EPI_ERR_CAPACITY and a message from
 * epi_engine_last_error(NULL) -- e.g. 1,000,000 agents on a 2,500 grid fit (29 MB),
 * 1,000,000 agents on a 3,500 grid (53 MB) do not.
 *
 * Arrays (device pointers, n = params->number_of_agents, G = params->grid_size), in the
 * engine's packed layout, updated in place:
 *   pos[n]            x | y << 16
 *   state[2n]         per agent: word 0 = disease state (bits 0-2), hospitalized (3),
 *                     isolated (4), vaccinated (5), work-quarantined (6), public transport (7),
 *                     current-area code (8-10: 0 home, 1 office, 2 transport strip, 3 housing
 *                     strip, 4 hospital, 5 grown hospital), work status (11-12), immunity + 2
 *                     (13-15), infection day (16-31); word 1 = at_hour.  8-byte aligned.
 *   home[n], work[n]  start corners of the 2x2 house / 10x10 office, packed like pos (read only)
 *   work_start_at[n]  hospital staff schedule
 * pos, home, work, work_start_at and counts must be 4-byte aligned.
 *   plane[(G+3)^2+16] one byte per cell with a one-cell border: cell (x, y) at
 *                     (y+1)*(G+3) + x+1; 0 vacant, 1 occupied, 2/3 infectious at the regular /
 *                     high rate; border and slack bytes zero.  4-byte aligned.
 *   counts[8]         out: S, E, I, H, R, D of this hour in counts[0..5]
 * hospital_grown = 1 once BuildNewHospital has fired.  The call is issued on cuda_stream
 * (NULL = the legacy default stream) and returns after the hour has finished.  The first call
 * on a device looks up the scratch array's device address and the launch shape while that
 * device is current; make it before any stream capture.  Every call shares the scratch array
 * and starts by clearing the parts that must start clean, so calls in a row are independent;
 * calls whose work overlaps on the GPU (other streams, other host threads) race on it. */
int epi_tick_hour_noalloc(const epi_params* params, uint32_t hour, uint32_t hospital_grown, uint32_t* pos,
                          uint32_t* state, const uint32_t* home, const uint32_t* work, uint32_t* work_start_at,
                          uint8_t* plane, uint32_t* counts, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* EPI_ENGINE_H */
