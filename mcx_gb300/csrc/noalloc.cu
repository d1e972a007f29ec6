// noalloc.cu -- a transport entry point that allocates no device memory.
//
// Who needs it: callers that are not allowed to call cudaMalloc once they are running -- a host
// application that owns every byte of device memory through its own pool and hands the engine
// only buffers it carved out itself, or a latency-critical loop where cudaMalloc's implicit
// device synchronisation is unacceptable.  Such a caller allocates the labels, the two field
// accumulators and the detected-photon buffer up front and passes them in; the few bytes of
// bookkeeping the kernel needs besides those (photon counter, step/deposit counters, FP64
// energy tallies, error word, detected-photon counter, detector table) live in the static
// device array below instead of being allocated per call.
//
// The array is a file-scope `__device__` object: every process that loads libmcx_gb300.so keeps
// kScratchBytes of it on each GPU it uses until it exits.  All calls share it and it keeps the
// last call's contents, so each call clears what has to start at zero; two calls that overlap
// on the GPU (different streams, or different host threads on one device) race on it and must
// be serialised by the caller.

#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/mcx_abi.h"
#include "../../include/mcx_gb300.h"
#include "mcxg_common.h"
#include "transport.cuh"

namespace mcxg {
namespace {

// Layout of the static scratch: counters, tallies, words, then the detector table.
constexpr size_t kOffWork = 0;                                               // 1 x u64
constexpr size_t kOffCounters = 64;                                          // kNumCounters x u64
constexpr size_t kOffEnergy = kOffCounters + 8 * kNumCounters;               // kNumEnergy x f64
constexpr size_t kOffErr = kOffEnergy + 8 * kNumEnergy;                      // u32
constexpr size_t kOffDetCount = kOffErr + 4;                                 // u32
constexpr size_t kOffDetPos = 256;                                           // kMaxDetectors x float4
constexpr size_t kScratchBytes = kOffDetPos + sizeof(float4) * kMaxDetectors;
static_assert(kOffDetCount + 4 <= kOffDetPos, "scratch layout overlaps");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once per device).
unsigned char* scratch_for(int device) {
    if (device < 0 || device >= kMaxDevices) MCXG_RAISE(-6, "device index out of range for the allocation-free entry point");
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) MCXG_RAISE(-(int)e, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        g_scratch_ptr[device] = p;
    }
    return static_cast<unsigned char*>(g_scratch_ptr[device]);
}

// Kernel parameters of a prepared Config (the same values Session::create derives in
// engine.cu), without touching device memory.
void fill_kparams(const Config* cfg, KParams& k, bool& reflect, bool& savedet) {
    std::memset(&k, 0, sizeof(k));
    const size_t nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
    int totalgates = (int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5f);
    if (totalgates < 1) totalgates = 1;
    k.nx = (int)cfg->dim.x; k.ny = (int)cfg->dim.y; k.nz = (int)cfg->dim.z;
    k.dimxy = cfg->dim.x * cfg->dim.y;
    k.nvox = (unsigned)nvox;
    k.medianum = (int)cfg->medianum;
    for (unsigned i = 0; i < cfg->medianum; i++)
        k.prop[i] = make_float4(cfg->prop[i].mua, cfg->prop[i].mus, cfg->prop[i].g, cfg->prop[i].n);
    k.oneoverc0 = kR_C0 * cfg->unitinmm;
    k.Rtstep = 1.f / cfg->tstep;
    k.maxgate = (cfg->maxgate > 0) ? std::min<int>((int)cfg->maxgate, totalgates) : totalgates;
    k.doreflect = cfg->isreflect ? 1 : 0;
    k.save2pt = cfg->issave2pt ? 1 : 0;
    k.saveref = (cfg->issave2pt && cfg->issaveref == 1) ? 1 : 0;
    k.outputtype = cfg->outputtype;
    if (k.outputtype != otFlux && k.outputtype != otFluence && k.outputtype != otEnergy)
        MCXG_RAISE(-6, "the allocation-free entry point supports flux, fluence and energy outputs");
    if (cfg->mediabyte > 4)
        MCXG_RAISE(-6, "the allocation-free entry point takes byte labels: no per-voxel media formats");
    if (cfg->seed == kSEED_FROM_FILE || cfg->issaveseed)
        MCXG_RAISE(-6, "the allocation-free entry point runs no replay and saves no seeds");
    if (cfg->polmedianum)
        MCXG_RAISE(-6, "the allocation-free entry point runs no polarised media (they need a Mueller table buffer)");
    if (cfg->debuglevel & (kDebugMove | kDebugMoveOnly))
        MCXG_RAISE(-6, "the allocation-free entry point saves no trajectories (they need a record buffer)");
    if (cfg->extrasrclen)
        MCXG_RAISE(-6, "the allocation-free entry point runs one source (extra sources need a device buffer)");
    if (cfg->issaveref)
        MCXG_RAISE(-6, "the allocation-free entry point records no diffuse reflectance");
    if (cfg->nphase > 2 || cfg->nangle)
        MCXG_RAISE(-6, "the allocation-free entry point takes no phase-function or launch-angle tables (they need device buffers)");
    k.minenergy = cfg->minenergy;
    k.gscatter = (float)cfg->gscatter;
    k.maxvoidstep = (float)cfg->maxvoidstep;
    std::memcpy(k.bc, cfg->bc, 12);
    reflect = cfg->isreflect != 0;
    for (int i = 0; i < 6; i++)
        if (cfg->bc[i] == BC_REFLECT || cfg->bc[i] == BC_MIRROR) reflect = true;
    bool bcdet = false;
    for (int i = 6; i < 12; i++) bcdet = bcdet || cfg->bc[i] != 0;
    savedet = cfg->issavedet && (cfg->detnum > 0 || bcdet);
    const unsigned f = cfg->savedetflag;
    k.savedetflag = f;
    k.nmedia_det = (int)cfg->medianum - 1;
    k.partialdata = (cfg->medianum - 1) * (((f >> 1) & 1u) + ((f >> 2) & 1u) + ((f >> 3) & 1u));
    k.reclen = k.partialdata + (f & 1u) + 3u * (((f >> 4) & 1u) + ((f >> 5) & 1u)) + ((f >> 6) & 1u);
    k.maxdet = cfg->maxdetphoton;
    k.ndet = (int)cfg->detnum;

    fill_source(k, cfg, nullptr);
    k.step_cap = current_step_cap();
    k.chunk = 64;

    // shared-memory deposit tile over the entry point, as the session places it by default
    place_tile(k, 16);
}

// Sets kErrBadLabel in *err when a voxel's label (bits 0-6) is not below medianum: the kernel
// would read such a label's properties past the end of the medium table.
__global__ void check_labels_kernel(const uint8_t* __restrict__ labels, size_t n, unsigned medianum, unsigned* err) {
    bool bad = false;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        bad |= (unsigned)(labels[i] & kLabelMask) >= medianum;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(err, (unsigned)kErrBadLabel);
}

#define NCK(call)                                                                \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) MCXG_RAISE(-(int)e_, cudaGetErrorString(e_));    \
    } while (0)

void run_noalloc(const Config* cfg, const uint8_t* d_labels, float* d_field, float* d_spill, float* d_detp,
                 uint64_t photon_offset, uint64_t nphoton, int gate_group, cudaStream_t stream, mcxg_stats* stats) {
    if (!cfg || !d_labels || !d_field || !d_spill) MCXG_RAISE(-4, "labels, field and spill buffers are required");
    if (cfg->srctype == kSrcPattern || cfg->srctype == kSrcPattern3D)
        MCXG_RAISE(-6, "pattern sources need a device pattern buffer, which the allocation-free entry point does not take");
    if (cfg->medianum < 1 || cfg->medianum > (unsigned)kMaxMedia) MCXG_RAISE(-6, "the GB300 engine supports 1 to 128 media labels");
    if (cfg->detnum > (unsigned)kMaxDetectors)
        MCXG_RAISE(-6, "the allocation-free entry point holds at most 256 detectors in its static scratch");
    if (cfg->dim.x >= 32768 || cfg->dim.y >= 32768 || cfg->dim.z >= 32768) MCXG_RAISE(-6, "volume dimensions must be below 32768");
    if (current_seeding_mode() == 1)
        MCXG_RAISE(-6, "the allocation-free entry point runs per-photon RNG streams only: MCX seeding (mcxg_set_seeding(1) or "
                       "MCXG_SEEDING=mcx) needs a device buffer of per-thread seed words");
    int device = 0;
    NCK(cudaGetDevice(&device));
    unsigned char* s = scratch_for(device);

    KParams k;
    bool reflect = false, savedet = false;
    fill_kparams(cfg, k, reflect, savedet);
    if (savedet && !d_detp) MCXG_RAISE(-4, "a detected-photon buffer is required when detectors are saved");
    const float twin0 = cfg->tstart + cfg->tstep * (float)k.maxgate * (float)gate_group;
    k.twin0 = twin0;
    k.twin1 = twin0 + cfg->tstep * (float)k.maxgate;
    k.labels = d_labels;
    k.field = d_field;
    k.shadow = d_spill;
    k.field64 = nullptr;
    k.detp = savedet ? d_detp : nullptr;
    k.work = reinterpret_cast<unsigned long long*>(s + kOffWork);
    k.counters = reinterpret_cast<unsigned long long*>(s + kOffCounters);
    k.energy = reinterpret_cast<double*>(s + kOffEnergy);
    k.errflag = reinterpret_cast<unsigned*>(s + kOffErr);
    k.detcount = reinterpret_cast<unsigned*>(s + kOffDetCount);
    k.detpos = reinterpret_cast<const float4*>(s + kOffDetPos);
    k.photon_offset = photon_offset;
    k.nphoton = nphoton;
    k.seed = (uint64_t)(uint32_t)cfg->seed;

    // the array keeps the previous call's values: clear every accumulator, then the detectors
    NCK(cudaMemsetAsync(s, 0, kOffDetPos, stream));
    if (cfg->detnum)
        NCK(cudaMemcpyAsync(s + kOffDetPos, cfg->detpos, sizeof(float4) * cfg->detnum, cudaMemcpyHostToDevice, stream));

    int sms = 0;
    NCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    // every label must index the medium table: checked on the device before any photon runs
    unsigned words[2] = {0u, 0u};
    check_labels_kernel<<<4 * sms, 256, 0, stream>>>(d_labels, (size_t)k.nvox, (unsigned)k.medianum,
                                                     reinterpret_cast<unsigned*>(s + kOffErr));
    NCK(cudaGetLastError());
    NCK(cudaMemcpyAsync(words, s + kOffErr, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    NCK(cudaStreamSynchronize(stream));
    if (words[0] & kErrBadLabel) MCXG_RAISE(-4, "input media optical properties are less than the labels in the volume");

    // launch shape as the session picks it: without room for the deposit tile, run without it
    const int block = 256;
    size_t smem = transport_smem_bytes(k, block, savedet);
    int bps = transport_blocks_per_sm(reflect, savedet, transport_mode(k), block, smem);
    if (bps <= 0 && k.tile_on) {
        k.tile_on = 0;
        smem = transport_smem_bytes(k, block, savedet);
        bps = transport_blocks_per_sm(reflect, savedet, transport_mode(k), block, smem);
    }
    if (bps <= 0) MCXG_RAISE(-6, "the transport kernel does not fit on this device");
    NCK(launch_transport(k, reflect, savedet, bps * sms, block, smem, stream));

    // the error word and the detected count are always read back: a run stopped by the step cap
    // or the index guard fails even when the caller asks for no statistics
    double e[kNumEnergy];
    unsigned long long c[kNumCounters];
    if (stats) {
        NCK(cudaMemcpyAsync(e, s + kOffEnergy, sizeof(e), cudaMemcpyDeviceToHost, stream));
        NCK(cudaMemcpyAsync(c, s + kOffCounters, sizeof(c), cudaMemcpyDeviceToHost, stream));
    }
    NCK(cudaMemcpyAsync(words, s + kOffErr, sizeof(words), cudaMemcpyDeviceToHost, stream));
    NCK(cudaStreamSynchronize(stream));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->e_launch = e[kELaunch]; stats->e_escape = e[kEEscape]; stats->e_detect = e[kEDetect];
        stats->e_absdep = e[kEAbsDep]; stats->e_absother = e[kEAbsOther];
        stats->n_steps = c[kCntSteps]; stats->n_scatter = c[kCntScatter]; stats->n_deposit = c[kCntDeposit];
        stats->n_launch = c[kCntLaunch]; stats->n_photon = c[kCntPhoton]; stats->n_detected = words[1];
        stats->n_tile_deposit = c[kCntTileDeposit];
        stats->grid = bps * sms; stats->block = block; stats->chunk = k.chunk; stats->launches = 1;
        stats->error_flags = words[0];
    }
    if (words[0] & kErrStepCap) MCXG_RAISE(-6, "a photon exceeded the per-photon step cap; the simulation was stopped");
    if (words[0] & kErrIndex) MCXG_RAISE(-6, "internal error: a photon's voxel index left the volume; the photon was stopped");
}

}  // namespace
}  // namespace mcxg

using namespace mcxg;

// Allocation-free transport launch: see include/mcx_gb300.h for the contract.
extern "C" int mcxg_run_noalloc(const Config* cfg, const uint8_t* d_labels, float* d_field, float* d_spill, float* d_detp,
                                uint64_t photon_offset, uint64_t nphoton, int gate_group, void* stream, mcxg_stats* stats) {
    mcxg_clear_error();
    try {
        run_noalloc(cfg, d_labels, d_field, d_spill, d_detp, photon_offset, nphoton, gate_group,
                    static_cast<cudaStream_t>(stream), stats);
        return 0;
    } catch (const Error& e) {
        mcxg_set_error(e.id ? e.id : -1, e.msg.c_str());
        return e.id ? e.id : -1;
    }
}

extern "C" size_t mcxg_noalloc_scratch_bytes(void) { return kScratchBytes; }
