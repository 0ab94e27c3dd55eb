/*
 * emt6ro_gb300.h -- C ABI of the GB300-native EMT6-Ro batched simulator.
 *
 * Plain C types only (pointers, sizes, POD structs); every entry point returns
 * an int status (EMT6_OK = 0) and stores a message retrievable with
 * emt6_last_error() on failure.  Each entry point names the reference
 * interface it replaces (paths relative to the banasraf/EMT6-Ro project).
 *
 * Threading: calls on one handle must not run concurrently from several host
 * threads (the library takes a per-handle mutex and returns EMT6_ERR_STATE for
 * calls that conflict with a running experiment).  Device work is issued on
 * one CUDA stream per handle.
 */
#ifndef EMT6RO_GB300_H_
#define EMT6RO_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMT6_OK 0
#define EMT6_ERR_INVALID 1 /* bad argument */
#define EMT6_ERR_CUDA 2    /* CUDA runtime error */
#define EMT6_ERR_STATE 3   /* call not allowed now (e.g. already running) */
#define EMT6_ERR_IO 4      /* file missing or unparsable */
#define EMT6_ERR_LIMIT 5   /* size beyond a supported maximum */
#define EMT6_ERR_DEVICE 6  /* a kernel raised its error flag */

/* Largest lattice the kernels hold on chip: interior height <= 54 and
 * interior width <= 60 (the reference's diffusion tile stops at 55,
 * src/emt6ro/diffusion/diffusion.cu:13). */
#define EMT6_MAX_INTERIOR_HEIGHT 54
#define EMT6_MAX_INTERIOR_WIDTH 60
#define EMT6_INSTR_HIST_N 300 /* src/emt6ro/common/instr.h:41 */

/* Model parameters; same content as the reference's Parameters struct
 * (src/emt6ro/parameters/parameters.h:10-70), flattened. */
typedef struct {
  int32_t lattice_height, lattice_width; /* interior, border ring excluded */
  float time_step;                       /* seconds per step (6) */
  float diffusion_coeffs[3];             /* cho, ox, gi */
  float diffusion_time_step;             /* seconds per diffusion substep (0.25) */
  float metabolism[4][3]; /* aerobic prolif., anaerobic prolif., aerobic quiesc., anaerobic quiesc. */
  float external_levels[3];
  float death_gi, quiescence_gi, death_gi_production;
  float cycle_times[5][2]; /* (mean, stddev) for g1, s, g2, m, d */
  float delay_time_coeff, delay_time_exp_coeff;
  float survival_prob_coeff, survival_prob_exp_coeff;
  float repair_half_time;
} emt6_params;

/* One lattice site (replaces the reference's 56-byte Site, site/site.h:34-43).
 * state: 0 vacant, 1 occupied, 2 mocked border.  mode/phase: Cell enums
 * (cell/cell.h:18-26). */
typedef struct {
  float cho, ox, gi;
  float time_in_repair, irradiation, repair_delay_time, proliferation_time;
  float cycle_times[5];
  uint8_t mode, phase, state, pad;
} emt6_site;

typedef struct { /* src/emt6ro/common/instr.h:46-52 */
  unsigned long long repair_decisions, repair_kills, irradiation_events, divisions;
  double sum_death_prob;
} emt6_instr_counters;

typedef struct emt6_batch emt6_batch;
typedef struct emt6_experiment emt6_experiment;

/* Message of the last failing call on this host thread ("" if none). */
const char *emt6_last_error(void);
int emt6_version(void);

/* ---- file formats -------------------------------------------------------- */
/* Replaces Parameters::loadFromJSONFile (src/emt6ro/parameters/parameters.cc:66-80). */
int emt6_load_parameters(const char *path, emt6_params *out);
/* Replaces loadFromFile (src/emt6ro/state/state.cc:9-53).  Writes (H+2)*(W+2)
 * sites with the MOCKED border ring at the external levels; *height and *width are
 * the full dims.  Fails with EMT6_ERR_LIMIT if more than cap sites. */
int emt6_load_state(const char *path, const emt6_params *p, emt6_site *out, int32_t cap,
                    int32_t *height, int32_t *width);
/* Replaces saveToFile (src/emt6ro/state/state.cc:55-82). */
int emt6_save_state(const char *path, const emt6_site *sites, int32_t height, int32_t width);

/* ---- batch engine: any mix of tumours x protocols x horizons ---------------
 * Replaces Simulation (src/emt6ro/simulation/simulation.h:13-114):
 * constructor + sendData/setState + setProtocols.  n_tumors initial lattices
 * of height x width sites (border included) are kept once on the device;
 * simulation i starts from tumors[sim_tumor[i]], follows protocol
 * sim_protocol[i] (protocol_bins doses, one per protocol_resolution steps,
 * read while step < protocol_length) and stops at sim_horizon[i] (NULL = no
 * horizon).  seed keys the counter-based random stream. */
int emt6_batch_create(const emt6_params *p, const emt6_site *tumors, int32_t n_tumors,
                      int32_t height, int32_t width, int32_t n_protocols, uint32_t protocol_bins,
                      uint32_t protocol_resolution, uint32_t protocol_length, int64_t n_sims,
                      const int32_t *sim_tumor, const int32_t *sim_protocol,
                      const uint32_t *sim_horizon, int32_t device, uint64_t seed,
                      emt6_batch **out);
int emt6_batch_destroy(emt6_batch *b);
/* Restore the initial lattices, step counters to 0, protocol doses to 0; the
 * random stream moves to a fresh epoch (Simulation::reset + setState,
 * simulation.cu:212-223, and backend.cc:84-89). */
int emt6_batch_reset(emt6_batch *b);
/* doses[protocol * protocol_bins + bin] += dose for each (protocol, step, dose)
 * triple, bin = step / protocol_resolution (Protocol::closestDose,
 * src/emt6ro/common/protocol.h:16-18). */
int emt6_batch_add_irradiations(emt6_batch *b, const int32_t *protocol, const uint32_t *step,
                                const float *dose, int64_t n);
/* Overwrite all protocol doses (n_protocols * protocol_bins floats). */
int emt6_batch_set_doses(emt6_batch *b, const float *doses);
/* Enqueue nsteps simulation steps for every simulation (Simulation::run,
 * simulation.cu:193-198); returns without waiting. */
int emt6_batch_run(emt6_batch *b, uint32_t nsteps);
int emt6_batch_sync(emt6_batch *b);
/* Living-cell count per simulation after the enqueued work
 * (Simulation::getResults + countLiving, statistics.cu:9-38). Blocks. */
int emt6_batch_counts(emt6_batch *b, uint32_t *out);
/* Device-side summary after the enqueued work, 13 floats per simulation into
 * out[n][13]: cho, ox, gi at the centre site (H/2, W/2), living cells, living
 * cells per metabolic mode (4) and per cycle phase (5) -- the record of
 * example/timelapse.cc:24-45, without copying lattices to the host. Blocks. */
int emt6_batch_summary(emt6_batch *b, float *out);
/* Copy one simulation's lattice to the host (Simulation::getData, simulation.cu:200-206). */
int emt6_batch_get_state(emt6_batch *b, int64_t sim, emt6_site *out);
/* Current step counter of one simulation. */
int emt6_batch_step(emt6_batch *b, int64_t sim, uint32_t *out);
/* The batch's CUDA stream (cudaStream_t) for callers that time or order work. */
void *emt6_batch_stream(emt6_batch *b);
/* Diffused site-substeps executed since creation (for throughput accounting). */
int emt6_batch_diffused(emt6_batch *b, unsigned long long *out);
/* Kernels this handle has launched since creation (run, reset, count). */
int emt6_batch_launches(emt6_batch *b, unsigned long long *out);
/* Measured FP32 FMA throughput of the device (TFLOP/s): the ceiling the
 * FP32 stencil is reported against. No reference counterpart. */
int emt6_probe_fp32_peak(int32_t device, double *tflops);
/* Scheduling of emt6_batch_run.  mode bit 0: 0 = one CTA per simulation
 * (default), 1 = persistent CTAs taking simulations from a device work queue;
 * either way the simulations are taken largest diffusion region first, in an
 * order rebuilt on the device before every launch; bit 1: capture the run's launch sequence in
 * a CUDA graph and replay it (re-captured when start step, target, schedule,
 * chunk or epoch change).  steps_per_launch: steps per kernel launch (0 keeps
 * the current value, default 1200). */
int emt6_batch_set_schedule(emt6_batch *b, int32_t mode, uint32_t steps_per_launch);
/* Tile shapes the step kernels may use (the autotuner's second knob; every
 * shape gives bit-identical results): bit 0 = eight-lane bands for regions up
 * to 23 columns, bit 1 = three-column bands for 41-48-row regions of the wide
 * kernel, bit 2 = the 35 x 35 ring mapping on the narrow kernel; a cleared
 * bit falls back to the general layouts.  Default 7.  No reference
 * counterpart (its diffusion kernel has one tiling, diffusion.cu:135-191). */
int emt6_batch_set_layouts(emt6_batch *b, uint32_t layouts);
/* Key the random stream of simulation i by base + i (default base 0), so a
 * batch holding the contiguous shard [base, base + n_sims) of a larger set
 * draws exactly what one batch of the whole set would for those simulations
 * (sharding a GA population across GPUs without changing its results).  No
 * reference counterpart: the reference's curand streams follow its thread
 * layout (src/emt6ro/common/random-engine.cu:8-31). */
int emt6_batch_set_index_base(emt6_batch *b, uint32_t base);

/* ---- Experiment: protocols x tumours x runs ---------------------------------
 * Replaces the pybind11 _Experiment (python/emt6ro/simulation/backend.cc:16-136).
 * Simulation order is (protocol, tumour, run), as backend.cc:58-73. */
int emt6_experiment_create(const emt6_params *p, const emt6_site *tumors, int32_t n_tumors,
                           int32_t height, int32_t width, int32_t runs, int32_t protocols_num,
                           uint32_t simulation_steps, uint32_t protocol_resolution,
                           int32_t device, uint64_t seed, emt6_experiment **out);
int emt6_experiment_destroy(emt6_experiment *e);
/* backend.cc:91-101; protocol[i] in [0, protocols_num). */
int emt6_experiment_add_irradiations(emt6_experiment *e, const int32_t *protocol,
                                     const uint32_t *step, const float *dose, int64_t n);
/* backend.cc:103-113: EMT6_ERR_STATE if a run is pending. */
int emt6_experiment_run(emt6_experiment *e, uint32_t nsteps);
/* backend.cc:115-121: EMT6_ERR_STATE if no run is pending; out has
 * protocols_num * n_tumors * runs counts. Blocks. */
int emt6_experiment_results(emt6_experiment *e, uint32_t *out);
int emt6_experiment_reset(emt6_experiment *e); /* backend.cc:84-89 */
int emt6_experiment_state(emt6_experiment *e, int64_t sim, emt6_site *out); /* :123-134 */
emt6_batch *emt6_experiment_batch(emt6_experiment *e);

/* ---- instrumentation (src/emt6ro/common/instr.cu:6-48), per device -------- */
int emt6_read_instr_counters(int32_t device, emt6_instr_counters *out);
int emt6_reset_instr_counters(int32_t device);
/* 2 * EMT6_INSTR_HIST_N counts: irradiation histogram, then time-in-repair. */
int emt6_read_instr_histograms(int32_t device, unsigned long long *out);

/* ---- device unit hooks (run the library's device functions on given inputs;
 * used by the parity tests) --------------------------------------------------- */
int emt6_test_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out, int64_t n,
                     int32_t device);
int emt6_test_math(const float *x, float *expf_out, const double *u, double *log_out,
                   double *sin_out, double *cos_out, int64_t n, int32_t device);
int emt6_test_site_step(const emt6_params *p, emt6_site *sites, const uint32_t *vac,
                        const float *dose, const float *draws, int32_t *ready, int32_t *used,
                        int64_t n, int32_t device);
int emt6_test_choose(const float *u, int32_t r, int32_t c, int32_t *rc, int64_t n,
                     int32_t device);
int emt6_test_divide(const emt6_params *p, emt6_site *parents, const float *z,
                     emt6_site *children, int64_t n, int32_t device);
int emt6_test_normals(uint64_t seed, const uint32_t *step, const uint32_t *sim, uint32_t epoch,
                      float *z, int64_t n, int32_t device);
/* One step of ROI/list/diffusion building blocks on one lattice. */
int emt6_test_roi(const uint8_t *state, int32_t height, int32_t width, int32_t *roi,
                  uint8_t *mask, int32_t device);
int emt6_test_list(const uint8_t *state, int32_t height, int32_t width, uint16_t *list,
                   uint32_t *n, int32_t device);
/* variant 0: the narrow kernel's path (regions up to 32 x 31), 1: the wide one */
int emt6_test_diffuse(const emt6_params *p, float *fields, int32_t height, int32_t width,
                      const int32_t *roi, int32_t variant, int32_t device);
/* The launch order of a chunk ending at t_end for nsims simulations with
 * stored ROIs roi[8 i .. 8 i + 4] (r0, c0, h, w, dist), current steps and
 * optional horizons: order[] receives the simulation indices, largest region
 * first, simulations with nothing to do last. */
int emt6_test_order(const int32_t *roi, const uint32_t *step, const uint32_t *horizon,
                    int64_t nsims, uint32_t t_end, int64_t *order, int32_t device);

/* ---- allocation-free entry point -------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * code inside a host application or framework whose allocator owns all device
 * memory (a caching pool, or a host that fixes every device allocation at
 * start-up).  Every pointer argument except p is a DEVICE pointer the caller
 * owns: d_tumors (n_tumors x height x width emt6_site), d_sim_tumor /
 * d_sim_protocol (n_sims int32), d_doses (n_protocols x protocol_bins float)
 * and the output d_counts (n_sims uint32).  Runs nsteps steps of every
 * simulation from its initial lattice (random stream keyed by seed,
 * simulation index and epoch 0, so the counts equal those of emt6_batch_* on
 * the same inputs) on the given cudaStream_t on the current device, then
 * synchronises that stream and returns.
 * The working state lives in a fixed 8 MiB device array inside the library
 * (held by every GPU that loads it until exit): at most 47 simulations of the
 * default 53 x 53 lattice per call; larger requests fail with EMT6_ERR_LIMIT.
 * The first call on a device (and the first after its context is re-created)
 * looks the array's address up: make it before any stream capture.  All calls
 * share the array; calls that overlap on the GPU race on it, so serialise
 * them across streams and threads. */
int emt6_simulate_noalloc(const emt6_params *p, const emt6_site *d_tumors, int32_t height,
                          int32_t width, const int32_t *d_sim_tumor,
                          const int32_t *d_sim_protocol, int64_t n_sims, const float *d_doses,
                          uint32_t protocol_bins, uint32_t protocol_resolution,
                          uint32_t protocol_length, uint32_t nsteps, uint64_t seed,
                          uint32_t *d_counts, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* EMT6RO_GB300_H_ */
