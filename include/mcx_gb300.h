/*
 * mcx_gb300.h -- C-ABI of libmcx_gb300.so beyond the two MCX entry points.
 *
 * The drop-in boundary itself is mcx_run_simulation / mcx_list_gpu (include/mcx_abi.h),
 * replacing src/mcx_core.h:200-201 of MCX.  The functions below are what a front-end that
 * does not link MCX's own mcx_utils.c needs around them (Config defaults and preparation,
 * error retrieval), plus a device-resident session interface used for benchmarking and by
 * the batched scheduler.  All take plain pointers and sizes.
 */
#ifndef MCX_GB300_H
#define MCX_GB300_H

#include <stdint.h>
#include "mcx_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Config preparation (host only; no GPU needed) -------------------------------------- */

/* Default values of every Config field.
 * Replaces mcx_initcfg, src/mcx_utils.c:248-378 (the parentid default is mpPython). */
void mcxg_initcfg(Config* cfg);

/* Prepare a filled Config for mcx_run_simulation: origin shift of source and detectors,
 * time-gate checks, source-direction normalisation, boundary flags, unitinmm scaling,
 * mus==0 media, launch voxel in srcparam2.z/.w, detector masking.  Returns 0 or a negative
 * MCX error id (message via mcxg_last_error).
 * Replaces mcx_validatecfg + mcx_preprocess, src/mcx_utils.c:3748-3857 and 1525-1820, for the
 * label-media pencil-source subset the engine runs. */
int  mcxg_validatecfg(Config* cfg);

/* Set bit 31 of every voxel that a detector sphere covers on an interface.
 * Replaces mcx_maskdet, src/mcx_utils.c:4214-4340 (label media). */
void mcxg_maskdet(Config* cfg);

/* ---- Errors ------------------------------------------------------------------------------ */

/* When no front-end provides mcx_error() (src/mcx_utils.c:1314), the engine records its
 * error here instead of exiting; mcx_run_simulation then returns normally. */
const char* mcxg_last_error(void);
int         mcxg_last_error_id(void);
void        mcxg_clear_error(void);
void        mcxg_set_error(int id, const char* msg);

/* ---- Run statistics ---------------------------------------------------------------------- */

/* Everything the last mcx_run_simulation on this thread measured, beyond what Config holds:
 * FP64 energy tallies for the balance launched = absorbed + escaped + detected, the GPU's
 * own step / scatter / deposit counters, kernel time from CUDA events, launch shape. */
typedef struct mcxg_stats {
    double e_launch;          /* total launched packet weight */
    double e_escape;          /* residual weight of photons that left undetected or timed out */
    double e_detect;          /* residual weight of detected photons */
    double e_absdep;          /* absorbed weight recorded in the field */
    double e_absother;        /* absorbed weight outside the recorded time window */
    uint64_t n_steps, n_scatter, n_deposit, n_launch, n_photon, n_detected;
    uint64_t n_tile_deposit;  /* deposits absorbed by the per-CTA shared-memory tile */
    double kernel_ms;         /* transport kernels, CUDA events */
    double total_ms;          /* whole mcx_run_simulation call, host clock */
    int grid, block, chunk, launches;
    uint32_t error_flags;     /* device-side error word (0 = clean) */
} mcxg_stats;

int mcxg_get_stats(mcxg_stats* out);

/* ---- RNG test kernel --------------------------------------------------------------------- */

/* Run the xorshift128+ generator on the GPU from four 32-bit seed words and copy n floats
 * to host memory.  Replaces the -D R kernel mcx_test_rng, src/mcx_core.cu:1731-1742. */
int mcxg_rng_test(const uint32_t seeds[4], float* out, int n);

/* n floats of the per-photon stream of photon `pid` under `seed`, generated on the GPU. */
int mcxg_photon_stream(uint64_t seed, uint64_t pid, float* out, int n);

/* Measured FP32 reduction (atomicAdd without return) throughput into L2 over `nfloats`
 * distinct addresses, in reductions per second: the deposit-bound term of the transport
 * roofline, measured on the device in use. */
int mcxg_probe_atomic_rate(uint64_t nfloats, double* per_second);

/* ---- Device-resident sessions ------------------------------------------------------------ */

/* A prepared simulation held on one device: labels, properties, detectors and output
 * buffers are uploaded once; runs then launch only the transport kernel.  Used by the
 * benchmark (inputs resident in HBM) and by the batched scheduler. */
typedef struct mcxg_session mcxg_session;

mcxg_session* mcxg_session_create(const Config* cfg, int device);
/* Clear the fluence, detected-photon and tally buffers. */
int  mcxg_session_reset(mcxg_session* s);
/* Simulate photons [photon_offset, photon_offset + nphoton) with RNG seed `seed` into the
 * session's buffers (accumulating); kernel time in *kernel_ms when non-NULL. */
int  mcxg_session_run(mcxg_session* s, uint64_t photon_offset, uint64_t nphoton, uint64_t seed, float* kernel_ms);
/* Copy out the raw accumulated field (maxgate x Nvox floats, shadow copies merged) and
 * up to max_records detected records; returns the number of detected photons seen. */
int64_t mcxg_session_read(mcxg_session* s, float* field, float* detp, uint64_t max_records, mcxg_stats* stats);
void mcxg_session_destroy(mcxg_session* s);
/* Pick the session's deposit-tile size from short pilot launches sized for a run of `nphoton`
 * photons (cached per configuration for the process); clears the session's buffers.
 * mcx_run_simulation does this itself for runs of 2e7 photons or more unless MCXG_TUNE=0. */
int  mcxg_session_autotune(mcxg_session* s, uint64_t nphoton);

/* Launch-shape override used by the autotuner (0 = engine default). */
void mcxg_set_launch(int block, int blocks_per_sm, int chunk, int tile);

/* RNG seeding of sessions and runs created afterwards.  0 (default): every photon has its own
 * xorshift128+ stream derived from (seed, photon index) -- results independent of launch shape.
 * 1: MCX's scheme -- one stream per MCX GPU thread (the count MCX's autopilot picks for the
 * device), seeded with glibc rand() words after srand(seed), each stream running its share of
 * photons in sequence (src/mcx_core.cu:3014-3016, 3247-3251, 3381-3387); the same seed then gives
 * the same random streams as MCX itself.  The environment variable MCXG_SEEDING=mcx selects 1. */
void mcxg_set_seeding(int mode);

/* Restatement of mcx_replayinit (src/mcx_utils.c:3624-3690) for front-ends that do not link
 * mcx_utils.c: prepares a replay (cfg->seed == SEED_FROM_FILE) from the baseline run's detected
 * photons `detps` (dimdetps[1] records of dimdetps[0] floats, saved with savedetflag 'dp') and
 * their seeds in cfg->replay.seed (seedbyte bytes each, compacted in place): keeps the photons of
 * detector cfg->replaydet (all when <= 0) detected within [tstart, tend] and fills
 * cfg->replay.weight / tof / detid and cfg->nphoton.  Returns 0 or a negative MCX error id. */
int mcxg_replayinit(Config* cfg, const float* detps, const int dimdetps[2], int seedbyte);

/* Per-photon step cap of the simulations started after the call (0 restores the default 2e7).
 * A photon still running after that many steps (checked every 1024 steps of its GPU thread) is
 * stopped and the run fails with MCX error -6; it guards against inputs that would keep a
 * photon alive forever.  No counterpart in MCX. */
void mcxg_set_step_cap(unsigned int steps);

/* Field accumulation of the following mcx_run_simulation calls: 64 accumulates the fluence in
 * FP64 on the device (MCX's USE_DOUBLE build, src/mcx_core.cu:55-63, 2243-2263: one FP64 copy
 * instead of the two-copy FP32 spill; exportfield stays float, as in MCX), anything else restores
 * FP32.  The default is FP32, or FP64 when the environment variable MCXG_FIELD_FP64=1 is set when
 * the first simulation starts, so unmodified front-ends can select it without recompiling, as
 * MCX needs.  No counterpart in MCX, which fixes the choice at compile time. */
void mcxg_set_field_precision(int bits);

/* The photon split mcx_run_simulation uses over the devices listed in cfg->deviceid (1-based ids,
 * as mcx_list_gpu leaves them; the same device may appear more than once): offsets[d] and
 * counts[d] of each launch's n photons for device d, in proportion to cfg->workload, or to the
 * devices' core counts in gpu[] (1 each when gpu is NULL) when cfg->workload is all zero, which
 * it then receives, as src/mcx_core.cu:2980-3007 fills it.  Unlike MCX, which truncates every
 * share, the last device takes the remainder so the shares add up to n.  Returns the number of
 * devices, or a negative MCX error id (-1: an active device without workload).  Host-only. */
int mcxg_photon_shares(Config* cfg, const GPUInfo* gpu, uint64_t nphoton, uint64_t* offsets, uint64_t* counts);

/* mcx_run_simulation with the fluence accumulated in FP64 on the device instead of MCX's FP32
 * two-copy scheme: the reference-accuracy twin the FP32 accumulation error is stated against.
 * Same inputs, outputs and errors as mcx_run_simulation (src/mcx_core.h:200).  No counterpart
 * in MCX. */
void mcxg_run_simulation_fp64(Config* cfg, GPUInfo* gpu);

/* ---- Batched simulations ------------------------------------------------------------------ */

/* No counterpart in MCX, whose front-ends run one mcx_run_simulation per input (src/mcx.c:62-78).
 * Runs `count` prepared Configs (each after mcxg_validatecfg or mcx_validatecfg) on the device of
 * cfgs[0]->deviceid[0], as one CUDA graph of their transport launches over `nstreams` streams
 * (1..32), largest photon budget first, each launch's grid sized by its stream's share of the
 * photons (times an oversubscription of 1 or 2, or MCXG_BATCH_OVERSUB when set) so that the
 * launches of all streams run side by side and the block scheduler fills the SMs a finishing
 * launch frees.  Every Config receives exactly the outputs
 * mcx_run_simulation gives it (exportfield accumulated, exportdetected, energies, normaliser,
 * detected count); its `runtime` is the whole batch's graph time.  Repetitions (respin) and gate
 * groups run in waves, one graph per wave holding every Config's next (group, repetition).
 * `stats` (count entries) and `graph_ms` may be NULL.  Returns 0 or a negative MCX error id (message via mcxg_last_error). */
int mcxg_run_batch(Config** cfgs, int count, int nstreams, mcxg_stats* stats, double* graph_ms);

/* mcxg_run_batch with the fluence kept on the device: for every i with dev_fields[i] != NULL the
 * normalised field of cfgs[i] (the size of its exportfield, which is neither allocated nor written)
 * is stored into that device buffer, for a consumer on the GPU such as a denoiser; the other
 * outputs are as mcxg_run_batch gives them.  Such a Config must save a field and run in one
 * repetition of one gate group, with one source pattern and no per-detector replay blocks.  The
 * buffers are complete when the call returns. */
int mcxg_run_batch_device(Config** cfgs, int count, int nstreams, float* const* dev_fields, mcxg_stats* stats,
                          double* graph_ms);

/* ---- Allocation-free transport ----------------------------------------------------------- */

/* No counterpart in MCX: an addition for callers that may not call cudaMalloc while they run,
 * such as an application that owns all device memory through its own pool, or a latency-bound
 * loop that cannot afford cudaMalloc's implicit device synchronisation.
 *
 * One transport launch over photons [photon_offset, photon_offset + nphoton) of the prepared
 * Config `cfg` (mcxg_validatecfg or MCX's mcx_validatecfg), time-gate group `gate_group`, on
 * `stream` (a cudaStream_t; NULL = legacy default stream) of the current device.  The caller
 * owns every buffer: d_labels (Nvox bytes, bit 7 = detector mask, bits 0-6 = medium label, every
 * label below cfg->medianum), d_field and d_spill (G x Nvox floats each, zeroed by the caller
 * before the first call; the fluence is their sum, unnormalised), d_detp (maxdetphoton x reclen
 * floats; may be NULL when no detectors are saved).  G, the gates of one group, is
 * min(cfg->maxgate, T) when cfg->maxgate > 0 and T otherwise, with
 * T = max(1, (int)((tend - tstart) / tstep + 0.5f)) (no memory cap, unlike mcx_run_simulation).
 * Nothing is allocated: the photon counter, counters, FP64 energy tallies, error word and
 * detector table live in a static device array of mcxg_noalloc_scratch_bytes() bytes that every
 * GPU using the library keeps until the process exits.  Limits: at most 256 detectors.  The
 * first call on a device looks up that array's device address, so make it before any stream
 * capture.  Calls share the array and clear it on entry: calls that overlap on the GPU race and
 * must be serialised.  The call waits for `stream` twice: after checking the labels on the device
 * and after the launch, to read the error word back.  It returns -4 for a label at or above
 * cfg->medianum (before any photon runs) and -6 for a run stopped by the per-photon step cap
 * (mcxg_set_step_cap) or the voxel-index guard.  `stats` (may be NULL) receives energies,
 * counters, the error word and the detected-photon count, which the caller needs to know how
 * many records of d_detp are valid (records past maxdetphoton are dropped, as MCX drops them).
 * Rejected with -6: per-voxel media formats, replay and seed saving, polarised media,
 * trajectories, extra sources, pattern sources, diffuse reflectance, phase-function and
 * launch-angle tables, output types other than flux / fluence / energy, and MCX seeding
 * (mcxg_set_seeding(1) or MCXG_SEEDING=mcx), which need further device buffers.  Returns 0 or a
 * negative MCX error id (message via mcxg_last_error). */
int mcxg_run_noalloc(const Config* cfg, const uint8_t* d_labels, float* d_field, float* d_spill, float* d_detp,
                     uint64_t photon_offset, uint64_t nphoton, int gate_group, void* stream, mcxg_stats* stats);
size_t mcxg_noalloc_scratch_bytes(void);

#ifdef __cplusplus
}
#endif

#endif /* MCX_GB300_H */
