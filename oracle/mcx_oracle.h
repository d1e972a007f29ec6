/* mcx_oracle.h -- C interface of the CPU oracle (test infrastructure only; see mcx_oracle.cpp). */
#ifndef MCX_ORACLE_H
#define MCX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One preprocessed simulation: the same inputs the engine receives through Config after
 * mcx_preprocess/mcx_maskdet (positions in grid units, mua/mus already scaled by unitinmm,
 * bit 31 of vol = detector mask, src_idx/src_med = the launch voxel and its label). */
typedef struct OracleProblem {
    const uint32_t* vol;
    uint32_t dim[3];
    const float* prop;        /* medianum x {mua, mus, g, n} */
    uint32_t medianum;
    const float* detpos;      /* detnum x {x, y, z, r} */
    uint32_t detnum;
    float srcpos[4];          /* w = launch weight */
    float srcdir[4];
    uint32_t src_idx, src_med;
    float twin0, twin1, tstep;
    uint32_t maxgate;
    float unitinmm;
    int isreflect, isspecular, voidtime, maxvoidstep, save2pt, outputtype;
    float minenergy;
    uint32_t gscatter;
    char bc[12];
    int savedet;
    uint32_t savedetflag, maxdetphoton;
    uint64_t nphoton, photon_offset, seed;
    int nthreads;
    /* seed_mode 0: one xorshift128+ state per photon from (seed, photon index).
     * seed_mode 1: MCX's own scheme (src/mcx_core.cu:3014-3016, 3247-3251, 3381-3387): `mcx_threads`
     * streams seeded with glibc rand() words after srand(seed); stream i simulates
     * nphoton/mcx_threads photons (+1 for the first nphoton%mcx_threads streams) in sequence. */
    int seed_mode;
    uint32_t mcx_threads;
    /* source shape (MCX_SRC_* numbering, src/mcx_const.h:84-101); src_idx/src_med are the launch
     * voxel of point sources; srcpattern holds pattern / pattern3d intensities, x fastest */
    int srctype;
    float srcparam1[4], srcparam2[4];
    const float* srcpattern;
    /* MCX mediabyte: 1/2/4 label volumes; 96 and 98-104 per-voxel formats whose 32-bit words
     * encode the properties (src/mcx_const.h:72-80, decoded as src/mcx_core.cu:582-730); 97 split
     * voxels, two words per voxel (the first words of all voxels, then the second words) */
    int mediaformat;
    /* extra sources (src/mcx_core.cu:1217-1227): nextra x 16 floats, MCX's ExtraSrc layout
     * {pos (w = weight), dir (w = focal length), param1, param2}; srcid 0 / -1 draws each photon's
     * source (-1: one block of gates per source), srcid k >= 1 runs source k */
    const float* extrasrc;
    uint32_t nextra;
    int srcid;
} OracleProblem;

/* Outputs: raw (unnormalised) field in FP64, optional per-voxel deposit counts, detected
 * records, energy tallies and the algorithmic counters the roofline uses. */
typedef struct OracleResult {
    double* field;            /* maxgate x Nvox, accumulated (+=) */
    uint64_t* hits;           /* optional, same shape */
    float* detp;              /* optional, maxdetphoton x reclen */
    double e_launch, e_escape, e_detect, e_absdep, e_absother;
    uint64_t n_steps, n_scatter, n_deposit, n_launch, n_detected, n_photon, n_saved;
    uint32_t reclen;
    double seconds;
} OracleResult;

int  oracle_version(void);
int  oracle_run(const OracleProblem* problem, OracleResult* result);
void oracle_rng_kat(const uint32_t seeds[4], float* out, int n);
void oracle_photon_stream(uint64_t seed, uint64_t pid, float* out, int n);

#ifdef __cplusplus
}
#endif

#endif
