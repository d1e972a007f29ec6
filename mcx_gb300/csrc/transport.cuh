// transport.cuh -- parameters of the GB300 photon-transport kernel and its launch helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "mcxg_common.h"

namespace mcxg {

// Indices into the device counter array.
enum Counter : int {
    kCntSteps = 0, kCntScatter, kCntDeposit, kCntLaunch, kCntPhoton, kCntDetected, kCntTileDeposit, kCntWork, kNumCounters
    // kCntLaunch: photons whose launch was attempted; kCntPhoton: photons that entered the
    // medium (the rest missed the volume after maxvoidstep attempts)
};
// Source types, MCX's MCX_SRC_* numbering (src/mcx_const.h:84-101).
enum SrcType : int {
    kSrcPencil = 0, kSrcIsotropic, kSrcCone, kSrcGaussian, kSrcPlanar, kSrcPattern, kSrcFourier, kSrcArcsine,
    kSrcDisk, kSrcFourierX, kSrcFourierX2D, kSrcZGaussian, kSrcLine, kSrcSlit, kSrcPencilArray, kSrcPattern3D,
    kSrcHyperboloid, kSrcRing, kNumSrcTypes
};
// Per-voxel media formats (src/mcx_const.h:72-80, decoded as src/mcx_core.cu:582-730 does).
enum MediaFormat : int {
    kMediaAsgnF2H = 96, kMedia2LabelSplit = 97, kMedia2LabelMix = 98, kMediaLabelHalf = 99, kMediaAsF2H = 100, kMediaMuaFloat = 101,
    kMediaAsHalf = 102, kMediaAsgnByte = 103, kMediaAsShort = 104
};
__host__ __device__ constexpr bool media_words(int f) {
    return (f >= kMediaAsgnF2H && f <= kMedia2LabelMix) || (f >= kMediaLabelHalf && f <= kMediaAsShort);
}

// Launch-direction options of area sources, from srcdir.w (src/mcx_core.cu:1672-1710): 0 =
// along srcdir, a finite value = focal length, NaN = isotropic, -inf = Lambertian.
// MCX's output types (src/mcx_utils.h:70).
enum OutputType : int {
    kOutFlux = 0, kOutFluence, kOutEnergy, kOutJacobian, kOutWP, kOutDCS, kOutRF, kOutL, kOutRFmus, kOutWLTOF, kOutWPTOF
};
enum FocusMode : int { kFocusNone = 0, kFocusLength, kFocusIsotropic, kFocusLambertian };
// Point sources: the launch voxel is the host's (srcparam2.z/.w after preprocessing).
__host__ __device__ constexpr bool src_is_point(int t) {
    return t == kSrcPencil || t == kSrcIsotropic || t == kSrcCone || t == kSrcArcsine || t == kSrcZGaussian;
}
// Indices into the device FP64 energy array.
enum Energy : int { kELaunch = 0, kEEscape, kEDetect, kEAbsDep, kEAbsOther, kNumEnergy };
// Bits of the device error word.
// debuglevel bits (src/mcx_const.h:67-70) and the trajectory record length (MCX_DEBUG_REC_LEN, :82)
enum DebugBits : unsigned { kDebugRNG = 1u, kDebugMove = 2u, kDebugProgress = 4u, kDebugMoveOnly = 8u };
constexpr unsigned kTrajRecLen = 6;
constexpr int kNAngles = 1000;              // scattering-angle samples of a Mueller table (NANGLES)

enum ErrBits : uint32_t { kErrStepCap = 1u, kErrBadLabel = 2u, kErrDetOverflow = 4u, kErrIndex = 8u };

// Everything one transport launch needs.  Passed as a __grid_constant__ kernel parameter, so
// uniform reads come from the constant bank; the per-medium table is copied to shared memory
// at kernel start because lanes index it with divergent labels.
struct KParams {
    // --- buffers (device pointers)
    const uint8_t* labels;          // Nvox bytes: bit 7 detector mask, bits 0-6 medium label
    const uint32_t* words;          // per-voxel media formats: MCX's 32-bit voxel words instead
    int mediaformat;                // MCX mediabyte: 1/2/4 labels, kMedia* per-voxel formats
    const uint32_t* words2;         // MEDIA_ASGN_F2H / MEDIA_2LABEL_SPLIT: each voxel's second word
    float* field;                   // maxgate x Nvox raw flux accumulator
    float* shadow;                  // maxgate x Nvox spill copy (values moved out past kMaxAccum)
    double* field64;                // FP64 accumulator (reference-accuracy runs only), else null
    float* detp;                    // maxdet x reclen detected-photon records
    unsigned int* detcount;         // detected photons seen (may exceed maxdet)
    double* energy;                 // kNumEnergy FP64 tallies
    unsigned long long* counters;   // kNumCounters
    unsigned int* errflag;          // device error word
    const float4* detpos;           // ndet x {x, y, z, r}

    // --- geometry
    int nx, ny, nz;
    unsigned int dimxy, nvox;

    // --- launch state every photon starts from (pencil beam: after void skipping on the host)
    float4 src_p;                   // x, y, z, initial weight
    float4 src_v;                   // unit direction
    float src_t;                    // time already spent in the void
    unsigned int src_idx;           // launch voxel
    unsigned int src_label;         // its label byte (detector bit included)
    int src_fx, src_fy, src_fz;     // integer voxel coordinates of the launch voxel
    int src_ok;                     // 0: photons cannot enter the volume (all launches fail)

    // --- other source shapes (src/mcx_core.cu:1261-1640): sampled per photon on the device,
    //     void skipping and specular loss per photon as well
    int srctype;                    // MCX_SRC_* (0 = pencil, the fixed launch state above)
    float4 src_param1, src_param2;  // srcparam1, srcparam2
    float src_focal;                // srcdir.w when finite: focal length
    int src_focus;                  // kFocus*: what srcdir.w asks of the area sources
    const float* srcpattern;        // pattern (param1.w x param2.w) or pattern3d intensities
    int isspecular, voidtime;

    // --- polarised light (src/mcx_core.cu:298-352, 1909-1933): per-medium Mueller tables
    int polarized;                  // label media with sphere populations (polmedianum > 0)
    const float4* smatrix;          // (medianum - 1) x kNAngles (S11, S12, S33, S34)
    float4 srciquv;                 // launch Stokes vector

    // --- photon trajectories, MCX's -D M (savedebugdata, src/mcx_core.cu:427-442; records at launch
    //     1681-1687, scattering 2068-2074, mismatched faces 2435-2441, termination 1116-1122)
    float* traj;                    // traj_max x 6 floats: id (uint bits), x, y, z, weight, source id; null: off
    unsigned* traj_count;           // records written (may exceed traj_max; the rest is dropped)
    unsigned traj_max;

    // --- seed saving and photon replay (src/mcx_core.cu:375-377, 1203-1215, 2018-2066, 2207-2226)
    int saveseed;                   // store each detected photon's generator state at launch
    unsigned long long* seeddata;   // maxdet x 2 words (xorshift128+ state)
    int replay;                     // photons start from saved states (MCX's SEED_FROM_FILE)
    const unsigned long long* replay_seed;  // nphoton x 2 words
    const float* replay_w;          // detected weight of each replayed photon
    const float* replay_tof;        // its time of flight (s)
    const int* replay_detid;        // its detector id
    int replaydet;                  // -1: one field block of maxgate gates per detector
    int detnum;
    float omega;                    // RF replay: angular modulation frequency (rad/s)
    size_t rf_offset;               // RF replay: offset of the imaginary half of the field

    // --- time gates
    float twin0, twin1, Rtstep, oneoverc0;
    int maxgate;

    // --- media (mua, mus, g, n) per label, already scaled to grid units
    int medianum;
    float4 prop[kMaxMedia];

    // --- physics switches
    int doreflect;                  // cfg->isreflect
    int save2pt;                    // record the field
    int saveref;                    // diffuse reflectance: -w into the void voxel a photon ends in
    int srcnum;                     // photon sharing: patterns (field channels); 1 otherwise
    const float* invcdf;            // user phase function: inverse CDF of cos(theta), nphase values
    int nphase;                     // > 2 replaces Henyey-Greenstein
    const float* angleinvcdf;       // launch zenith angles / pi, inverse CDF, nangle values
    int nangle;                     // > 0: launch directions from the table
    const float4* extrasrc;         // extra sources: 5 float4 each (pos, dir, param1, param2, focus)
    int nextra;                     // number of extra sources (extrasrclen)
    int traj_reclen;                // trajectory record: 6 floats, 10 with the Stokes vector
    int srcid;                      // 1: primary only, > 1: that source, 0: all merged, -1: all, one block each
    int outputtype;                 // 0 flux, 1 fluence, 2 energy
    float minenergy;                // Russian roulette threshold (0 = off)
    float gscatter;                 // scattering events after which mus' replaces mus
    float maxvoidstep;              // offset used by the nextafter nudge
    unsigned char bc[12];           // boundary condition codes per face, then detector flags

    // --- detectors
    int ndet;
    unsigned int maxdet, reclen, partialdata, savedetflag;
    int nmedia_det;                 // medianum - 1: rows of the per-medium record blocks

    // --- work
    unsigned long long nphoton;     // photons in this launch
    unsigned long long photon_offset;  // global index of the first one (RNG stream id)
    unsigned long long seed;
    unsigned long long* work;       // photon counter the persistent warps draw chunks from
    int chunk;                      // photons per warp refill
    unsigned int step_cap;          // safety cap on steps per photon (error flag when hit)

    // --- RNG seeding: 0 = one stream per photon from (seed, photon index); 1 = MCX's scheme, one
    //     stream per MCX thread seeded with host words, photons split statically over streams
    int seed_mode;
    const uint32_t* mcx_words;      // 4 words per stream (seed_mode 1)
    unsigned int mcx_streams, mcx_per, mcx_odd;

    // --- per-CTA shared-memory deposit tile (voxel box x gate range)
    int tile_on;
    int tx0, ty0, tz0, tnx, tny, tnz, tg0, tng;

    // --- derived at launch by launch_transport() from the fields above (constant-bank operands)
    float d_inv_c0;                 // 1 / oneoverc0: time is carried in grid-length units
    float d_tw0, d_tw1;             // time window in grid-length units
    float d_bin_a, d_bin_b;         // gate index = floor(t * d_bin_a - d_bin_b)
    float d_fnx, d_fny, d_fnz;      // dimensions as floats
    float d_tx0, d_ty0, d_tz0, d_tx1, d_ty1, d_tz1;   // tile box as floats
    float d_n0;                     // refractive index of medium 0
    int d_gscat;                    // gscatter as an integer threshold
    unsigned long long d_nwork;     // work items in the pool: photons, or MCX streams
    float d_tile_scale;             // fixed-point units per unit of deposited weight in the tile
    float d_tile_flush;             // weight of kTileFlushUnits units
    unsigned d_tile_lo, d_tile_span;  // voxel-index range [lo, lo + span) holding the tile box
};

// Spill threshold of the two-copy accumulation (src/mcx_core.h:53, MAX_ACCUM).
constexpr float kMaxAccum = 1000.f;
// Smallest deposit tile kept over the launch point: the voxels there receive millions of
// equal first-flight deposits, which must not be summed directly into large FP32 values.
constexpr int kMinTileKB = 2;
// Fixed-point units a tile slot hands to the global field at once (32-bit slots).
constexpr unsigned kTileFlushUnits = 1u << 30;

// Place the deposit tile: a box of voxels x gates around the point where photons enter the
// medium, extending along the launch direction, in `kb` KB of 32-bit slots (off when nothing
// is saved or the source misses the volume).
void place_tile(KParams& k, int kb);

// Host-side launch of the transport kernel variant matching the flags.  smem_bytes is the
// dynamic shared memory per CTA; returns the CUDA error of the launch.
cudaError_t launch_transport(const KParams& p, bool reflect, bool savedet, int grid, int block,
                             size_t smem_bytes, cudaStream_t stream);
// Register-budget variant of the transport kernel: 4 (64 registers, 4 CTAs of 256 per SM) or
// 3 (up to 85 registers).
void set_transport_variant(int minb);
int transport_variant();
// Shared memory the kernel needs for a given block size and parameter set.
size_t transport_smem_bytes(const KParams& p, int block, bool savedet);
// Kernel variant of a parameter set: 0 = pencil beam with flux/fluence/energy output, 1 = other
// source shapes sampled per photon, 2 = replay, seed saving or the replay / path-length outputs,
// 3 = everything of 2 on a per-voxel media format.
int transport_mode(const KParams& p);
bool transport_general(const KParams& p);
// Occupancy-derived CTAs per SM for the chosen variant.
int transport_blocks_per_sm(bool reflect, bool savedet, int mode, int block, size_t smem_bytes);

// Source fields of KParams from a preprocessed Config: shape parameters, the pencil's launch
// state (void skipping traced on the host), the point sources' launch voxel.  d_pattern holds
// the pattern intensities on the device (source_pattern_len floats) or is null.
void fill_source(KParams& k, const struct MCXConfig* cfg, const float* d_pattern);
size_t source_pattern_len(const struct MCXConfig* cfg);
// Rejects source settings the engine does not run (MCX error -6).
void check_source(const struct MCXConfig* cfg);

// Process-wide settings of new simulations (engine.cu): the RNG seeding scheme (0 = per-photon
// streams, 1 = MCX's per-thread streams; mcxg_set_seeding or MCXG_SEEDING=mcx) and the per-photon
// step cap (mcxg_set_step_cap).
int current_seeding_mode();
unsigned current_step_cap();

// Void skipping of a pencil source launched outside the volume or in a 0 voxel, traced once on
// the host (engine.cu).  Returns the entry voxel or -1.
int host_skipvoid(const struct MCXConfig* cfg, float4& p, float3& v, float& t, int fd[3]);

cudaError_t launch_atomic_probe(float* buf, unsigned n, int iters, int grid, int block, cudaStream_t stream);
cudaError_t launch_rng_test(const uint32_t* d_seeds, float* d_out, int n, cudaStream_t stream);
cudaError_t launch_photon_stream(unsigned long long seed, unsigned long long pid, float* d_out, int n, cudaStream_t stream);
cudaError_t launch_labels_from_vol(const uint32_t* d_vol, uint8_t* d_labels, size_t n, unsigned int medianum,
                                   unsigned int* d_err, cudaStream_t stream);
cudaError_t launch_merge_field(float* out, const float* field, const float* shadow, const double* field64, size_t n,
                               float scale, int normalize_positive_only, cudaStream_t stream);

}  // namespace mcxg
