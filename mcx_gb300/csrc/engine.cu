// engine.cu -- host driver of the GB300 engine and the C-ABI entry points.
//
// mcx_run_simulation / mcx_list_gpu replace MCX's src/mcx_core.cu:2621-2726 and 2740-4110 with
// the same contract towards the front-ends (Config in, fluence / detected photons / energies /
// runtime out, errors through mcx_error) but a different inside: one persistent transport
// launch per (time-gate group x respin) on a private stream, all outputs merged and normalised
// on the device before a single copy back, FP64 energy tallies, stream-ordered allocations
// that are reused across calls.
//
// Config fields read: nphoton, seed, srctype, srcpos, srcdir, srcparam1, srcparam2, srcpattern,
// tstart, tstep, tend, steps, dim, medianum, prop, detnum, detpos, maxdetphoton, maxgate, respin,
// vol, isreflect, isnormalized, issavedet, issaveseed, issave2pt, isspecular, outputtype,
// minenergy, unitinmm, flog, maxvoidstep, voidtime, savedetflag, deviceid, parentid, gscatter,
// bc, replay, replaydet, mediabyte, debuglevel, maxjumpdebug, issaveref, srcnum, srcid,
// extrasrclen, srcdata, nphase, invcdf, nangle, angleinvcdf, polmedianum, smatrix, srciquv,
// istrajstokes, omega.
// Config fields written: exportfield (+=), exportdetected and seeddata (realloc), exportdebugdata
// and debugdatalen (trajectories), detectedcount,
// runtime, energytot, energyabs, energyesc, normalizer, his.{normalizer,detected,respin,colcount,
// seedbyte,...}, deviceid (compacted by mcx_list_gpu).

#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdlib.h>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mcx_abi.h"
#include "../../include/mcx_gb300.h"
#include "mcxg_common.h"
#include "transport.cuh"

// Provided by an MCX front-end (src/mcx_utils.c) when one is linked; absent otherwise.
extern "C" void mcx_error(const int id, const char* msg, const char* file, const int linenum) __attribute__((weak));
extern "C" void mcx_savedata(float* dat, size_t len, Config* cfg) __attribute__((weak));
extern "C" void mcx_savedetphoton(float* ppath, void* seeds, int count, int seedbyte, Config* cfg) __attribute__((weak));
extern "C" int omp_get_thread_num(void) __attribute__((weak));

namespace mcxg {

namespace {
thread_local int t_err_id = 0;
thread_local std::string t_err_msg;
thread_local mcxg_stats t_stats;

struct LaunchOverride {
    int block = 0, blocks_per_sm = 0, chunk = 0, tile = -1;
} g_override;
std::mutex g_override_mu;

// Autotuner results: deposit-tile budget (KB) per configuration signature.
std::mutex g_tune_mu;
std::vector<std::pair<std::string, int>> g_tune_cache;

// RNG seeding of new sessions: -1 = not chosen yet (environment MCXG_SEEDING=mcx selects MCX's
// per-thread streams), 0 = per-photon streams, 1 = MCX's per-thread streams.
int g_seeding = -1;

// Field accumulation of mcx_run_simulation: 0 = not chosen yet (environment MCXG_FIELD_FP64=1
// selects FP64), 32 = FP32 with MCX's two-copy spill, 64 = FP64 (MCX's USE_DOUBLE build).
int g_field_bits = 0;

// Per-photon step cap of new sessions (a photon longer than this is stopped and reported).
constexpr unsigned kDefaultStepCap = 20000000u;
unsigned g_step_cap = kDefaultStepCap;

int seeding_mode() {
    std::lock_guard<std::mutex> g(g_override_mu);
    if (g_seeding < 0) {
        const char* e = std::getenv("MCXG_SEEDING");
        g_seeding = (e && std::strcmp(e, "mcx") == 0) ? 1 : 0;
    }
    return g_seeding;
}
}  // namespace

[[noreturn]] void raise(int id, const std::string& msg, const char* file, int line) { throw Error{id, msg, file, line}; }

int current_seeding_mode() { return seeding_mode(); }

bool field_fp64() {
    std::lock_guard<std::mutex> g(g_override_mu);
    if (g_field_bits == 0) {
        const char* e = std::getenv("MCXG_FIELD_FP64");
        g_field_bits = (e && std::strcmp(e, "1") == 0) ? 64 : 32;
    }
    return g_field_bits == 64;
}

unsigned current_step_cap() {
    std::lock_guard<std::mutex> g(g_override_mu);
    return g_step_cap;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) MCXG_RAISE(-(int)e_, cudaGetErrorString(e_));            \
    } while (0)

namespace {

// Route an engine error to the front-end's mcx_error (which exits or throws, as MCX does) or,
// without a front-end, record it for mcxg_last_error().
void report(const Error& e) {
    t_err_id = e.id ? e.id : -1;
    t_err_msg = e.msg;
    if (mcx_error) mcx_error(t_err_id, e.msg.c_str(), e.file, e.line);
}

// A device allocation released at scope exit, stream-ordered so the pool reuses it.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t s = nullptr;
    void alloc(size_t n, cudaStream_t stream) {
        release();
        s = stream;
        bytes = n;
        if (n) CK(cudaMallocAsync(&p, n, stream));
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        bytes = 0;
    }
    ~DevBuf() { release(); }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

float3 f3(float x, float y, float z) { return make_float3(x, y, z); }

// IEEE 754 binary16 bits to float (normals, subnormals, zero)
float half_to_float(uint32_t h) {
    const uint32_t sign = (h >> 15) & 1u, e = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
    const float v = e ? std::ldexp((float)(man | 0x400u), (int)e - 25) : std::ldexp((float)man, -24);
    return sign ? -v : v;
}

// Refractive index of voxel `id` (at grid coordinates f[3]) for a photon at p, as the kernel
// decodes it (props_of and split_voxel_at in transport.cu)
float host_n(const Config* cfg, long id, const int f3[3], const float4& p) {
    const uint32_t w = cfg->vol[id] & kMED_MASK;
    const int f = (int)cfg->mediabyte;
    if (!media_words(f) || w == 0) return cfg->prop[w].n;
    if (f == kMedia2LabelSplit) {
        const size_t nv = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        const uint32_t wb = cfg->vol[nv + id];
        const uint32_t lo = w >> 24, up = (w >> 16) & 0xFFu;
        float nx = ((wb >> 16) & 0xFFu) * (2.f / 255.f) - 1.f, ny = ((wb >> 8) & 0xFFu) * (2.f / 255.f) - 1.f,
              nz = (wb & 0xFFu) * (2.f / 255.f) - 1.f;
        if (up == 0 || nx * nx + ny * ny + nz * nz <= 0.f) return cfg->prop[lo].n;
        const float rx = ((w >> 8) & 0xFFu) * (1.f / 255.f) + f3[0], ry = (w & 0xFFu) * (1.f / 255.f) + f3[1],
                    rz = (wb >> 24) * (1.f / 255.f) + f3[2];
        return ((rx - p.x) * nx + (ry - p.y) * ny + (rz - p.z) * nz < 0.f) ? cfg->prop[up].n : cfg->prop[lo].n;
    }
    if (f == kMediaLabelHalf) return ((w >> 14) & 3u) == 3u ? std::fabs(half_to_float(w >> 16)) : cfg->prop[w & 0x3FFFu].n;
    if (f == kMedia2LabelMix) return cfg->prop[w & 0xFFu].n;     // the first tissue's, as the kernel's void search
    if (f == kMediaAsgnF2H) {
        const size_t nv = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        return std::fabs(half_to_float(cfg->vol[nv + id] >> 16));
    }
    if (f == kMediaAsgnByte) return (w >> 24) * (1.f / 127.f) * (cfg->prop[2].n - cfg->prop[1].n) + cfg->prop[1].n;
    return cfg->prop[1].n;
}

}  // namespace

// Void skipping of a pencil source launched outside the volume or in a 0 voxel
// (src/mcx_core.cu:866-956).  The path is deterministic, so the host traces it once and every
// photon starts from the result.  Returns the entry voxel or -1.
int host_skipvoid(const Config* cfg, float4& p, float3& v, float& t, int fd[3]) {
    const float mx = (float)cfg->dim.x, my = (float)cfg->dim.y, mz = (float)cfg->dim.z;
    const float minaccum = kR_C0 * cfg->unitinmm;
    const float rv[3] = {1.f / v.x, 1.f / v.y, 1.f / v.z};
    auto inside = [&](const int f[3]) {
        return (unsigned short)f[0] < mx && (unsigned short)f[1] < my && (unsigned short)f[2] < mz;
    };
    auto index = [&](const int f[3]) { return (long)f[2] * cfg->dim.x * cfg->dim.y + (long)f[1] * cfg->dim.x + f[0]; };
    int f[3] = {(int)std::floor(p.x), (int)std::floor(p.y), (int)std::floor(p.z)};
    int count = 1;
    while (true) {
        if (inside(f) && (cfg->vol[index(f)] & kMED_MASK)) {
            p.x -= v.x; p.y -= v.y; p.z -= v.z;
            f[0] = (int)std::floor(p.x); f[1] = (int)std::floor(p.y); f[2] = (int)std::floor(p.z);
            t -= minaccum;
            count = 0;
            int axis = -1;
            while (!inside(f) || !(cfg->vol[index(f)] & kMED_MASK)) {
                const float h0 = std::fabs((f[0] + (v.x > 0.f) - p.x) * rv[0]);
                const float h1 = std::fabs((f[1] + (v.y > 0.f) - p.y) * rv[1]);
                const float h2 = std::fabs((f[2] + (v.z > 0.f) - p.z) * rv[2]);
                const float d = std::fmin(std::fmin(h0, h1), h2);
                axis = (d == h0) ? 0 : ((d == h1) ? 1 : 2);
                t += minaccum * d;
                p.x += d * v.x; p.y += d * v.y; p.z += d * v.z;
                if (axis == 0) f[0] += (v.x > 0.f ? 1 : -1);
                if (axis == 1) f[1] += (v.y > 0.f ? 1 : -1);
                if (axis == 2) f[2] += (v.z > 0.f ? 1 : -1);
                if (count++ > 3) break;
            }
            if (!inside(f)) return -1;
            t = cfg->voidtime ? t : 0.f;
            const long id = index(f);
            const float n2 = host_n(cfg, id, f, p);
            if (cfg->isspecular && axis >= 0 && n2 != cfg->prop[0].n) {
                // specular loss at the entry face (reflectcoeff, src/mcx_core.cu:552-570) and refraction
                const float n1 = cfg->prop[0].n;
                const float vv[3] = {v.x, v.y, v.z};
                const float Icos = std::fabs(vv[axis]);
                const float a = n1 * n1, b = n2 * n2;
                float c = 1.f - a / b * (1.f - Icos * Icos);
                float R = 1.f;
                if (c > 0.f) {
                    float Re = a * Icos * Icos + b * c;
                    c = std::sqrt(c);
                    const float Im = 2.f * n1 * n2 * Icos * c;
                    R = (Re - Im) / (Re + Im);
                    Re = b * Icos * Icos + a * c * c;
                    R = (R + (Re - Im) / (Re + Im)) * 0.5f;
                }
                p.w *= 1.f - R;
                if (p.w > kEPS) {
                    float w3[3] = {v.x * n1 / n2, v.y * n1 / n2, v.z * n1 / n2};
                    const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
                    const float s = w3[a1] * w3[a1] + w3[a2] * w3[a2];
                    w3[axis] = (s < 1.f) ? std::sqrt(1.f - s) * (float)((w3[axis] > 0.f) - (w3[axis] < 0.f)) : 0.f;
                    const float r = 1.f / std::sqrt(w3[0] * w3[0] + w3[1] * w3[1] + w3[2] * w3[2]);
                    v = f3(w3[0] * r, w3[1] * r, w3[2] * r);
                }
            }
            fd[0] = f[0]; fd[1] = f[1]; fd[2] = f[2];
            return (int)id;
        }
        if ((p.x < 0.f && v.x <= 0.f) || (p.x >= mx && v.x >= 0.f) || (p.y < 0.f && v.y <= 0.f) ||
            (p.y >= my && v.y >= 0.f) || (p.z < 0.f && v.z <= 0.f) || (p.z >= mz && v.z >= 0.f))
            return -1;
        p.x += v.x; p.y += v.y; p.z += v.z;
        f[0] = (int)std::floor(p.x); f[1] = (int)std::floor(p.y); f[2] = (int)std::floor(p.z);
        t += minaccum;
        if (count++ > cfg->maxvoidstep) return -1;
    }
}

namespace {

// Byte-label volume of the host uint32 volume (bit 31 -> bit 7).  Done on the device when the
// session uploads; this host twin serves the void-skipping trace only.
uint32_t host_label(const Config* cfg, long id) { return cfg->vol[id]; }

}  // namespace

// Source settings the engine takes (src/mcx_core.cu:1261-1640): every MCX_SRC_* shape with one
// source or several (extrasrclen), photon sharing (srcnum > 1 patterns of a pattern source) and
// launch-angle tables.
void check_source(const Config* cfg) {
    if ((unsigned char)cfg->srctype >= kNumSrcTypes) MCXG_RAISE(-6, "unknown source type");
    if (std::isinf(cfg->srcdir.w) && cfg->srcdir.w > 0.f)
        MCXG_RAISE(-4, "a focal length of +inf is not a valid source setting (srcdir.w)");
    if (cfg->srcnum > 1) {
        const int t = (unsigned char)cfg->srctype;
        if (t != kSrcPattern && t != kSrcPattern3D)
            MCXG_RAISE(-6, "photon sharing (srcnum > 1) needs a pattern or pattern3d source");
        if (cfg->seed == kSEED_FROM_FILE || (cfg->outputtype != otFlux && cfg->outputtype != otFluence && cfg->outputtype != otEnergy))
            MCXG_RAISE(-6, "photon sharing is supported with flux, fluence and energy outputs, without replay");
    }
    if (cfg->extrasrclen) {              // src/mcx_utils.c:1679-1692
        if (!cfg->srcdata) MCXG_RAISE(-4, "extrasrclen is set but the extra sources (srcdata) are missing");
        if (cfg->srcnum > 1) MCXG_RAISE(-4, "simulating multiple sources currently can not be used with photon-sharing");
        if (cfg->srcid > (int)cfg->extrasrclen + 1) MCXG_RAISE(-4, "srcid exceeds total defined source count");
        for (unsigned i = 0; i < cfg->extrasrclen; i++)
            if (std::isinf(cfg->srcdata[i].srcdir.w) && cfg->srcdata[i].srcdir.w > 0.f)
                MCXG_RAISE(-4, "a focal length of +inf is not a valid source setting (srcdir.w)");
    }
    if (cfg->nangle && !cfg->angleinvcdf) MCXG_RAISE(-4, "nangle is set but the launch-angle table (angleinvcdf) is empty");
    if (cfg->nphase > 2 && !cfg->invcdf) MCXG_RAISE(-4, "nphase is set but the phase-function table (invcdf) is empty");
    const int st = (unsigned char)cfg->srctype;
    if ((st == kSrcPattern || st == kSrcPattern3D) && !cfg->srcpattern)
        MCXG_RAISE(-4, "the 'srcpattern' field can not be empty when your 'srctype' is 'pattern'");
    // pattern sizes index the pattern array: whole numbers of pixels / voxels
    auto whole = [](float x) { return x >= 1.f && x == std::floor(x) && x < 16777216.f; };
    if (st == kSrcPattern && !(whole(cfg->srcparam1.w) && whole(cfg->srcparam2.w)))
        MCXG_RAISE(-4, "a pattern source needs whole pattern dimensions in srcparam1.w and srcparam2.w");
    if (st == kSrcPattern3D && !(whole(cfg->srcparam1.x) && whole(cfg->srcparam1.y) && whole(cfg->srcparam1.z)))
        MCXG_RAISE(-4, "a pattern3d source needs whole pattern dimensions in srcparam1.x/y/z");
    if (st == kSrcPencilArray && !(cfg->srcparam1.w >= 2.f && cfg->srcparam2.w >= 2.f))
        MCXG_RAISE(-4, "a pencil-array source needs at least 2 beams along each side (srcparam1.w, srcparam2.w)");
}

// Field channels of a photon-sharing run: one per pattern (src/mcx_core.cu:2782); 1 otherwise.
unsigned share_channels(const Config* cfg) {
    const int t = (unsigned char)cfg->srctype;
    return (cfg->srcnum > 1 && (t == kSrcPattern || t == kSrcPattern3D)) ? cfg->srcnum : 1u;
}

size_t source_pattern_len(const Config* cfg) {
    if (!cfg->srcpattern) return 0;
    const size_t ns = share_channels(cfg);
    if ((unsigned char)cfg->srctype == kSrcPattern) return (size_t)cfg->srcparam1.w * (size_t)cfg->srcparam2.w * ns;
    if ((unsigned char)cfg->srctype == kSrcPattern3D) return (size_t)cfg->srcparam1.x * (size_t)cfg->srcparam1.y * (size_t)cfg->srcparam1.z * ns;
    return 0;
}

void fill_source(KParams& k, const Config* cfg, const float* d_pattern) {
    float4 p = cfg->srcpos;
    float3 v = f3(cfg->srcdir.x, cfg->srcdir.y, cfg->srcdir.z);
    float t = 0.f;
    k.srctype = (unsigned char)cfg->srctype;
    k.src_param1 = cfg->srcparam1;
    k.src_param2 = cfg->srcparam2;
    const float f = cfg->srcdir.w;
    k.src_focus = std::isnan(f) ? kFocusIsotropic
                : std::isinf(f) ? kFocusLambertian          // -inf; +inf is rejected by check_source
                : (f != 0.f) ? kFocusLength : kFocusNone;
    k.src_focal = std::isfinite(f) ? f : 0.f;
    k.srcpattern = d_pattern;
    k.srcnum = (int)share_channels(cfg);
    k.isspecular = cfg->isspecular ? 1 : 0;
    k.voidtime = cfg->voidtime;
    k.src_ok = 1;
    uint32_t sidx = 0, smed = 0;
    if (src_is_point(k.srctype)) {          // launch voxel from preprocessing (srcparam2.z/.w)
        std::memcpy(&sidx, &cfg->srcparam2.z, 4);
        std::memcpy(&smed, &cfg->srcparam2.w, 4);
    }
    int fd[3] = {(int)std::floor(p.x), (int)std::floor(p.y), (int)std::floor(p.z)};
    if (k.srctype == kSrcPencil && cfg->nangle == 0 && cfg->extrasrclen == 0) {
        // every pencil photon follows the same path through the void: traced once here, the
        // photons start from its end (src/mcx_core.cu:1236-1243, 1652-1672); with a launch-angle
        // table each photon has its own direction and the kernel launches it (MCX's non-pencil path)
        if ((smed & kMED_MASK) == 0) {
            const int id = host_skipvoid(cfg, p, v, t, fd);
            if (id < 0) {
                k.src_ok = 0;
            } else {
                sidx = (uint32_t)id;
                smed = host_label(cfg, id);
            }
        }
        if (std::fabs(p.w) <= cfg->minenergy) k.src_ok = 0;
    }
    k.src_p = p;
    k.src_v = make_float4(v.x, v.y, v.z, 0.f);
    k.src_t = t;
    k.src_idx = sidx;
    // byte-label form, or the raw word for the per-voxel media formats
    k.src_label = media_words(cfg->mediabyte) ? smed : ((smed & kLabelMask) | ((smed & kDET_MASK) ? kLabelDet : 0u));
    if (k.src_ok) {
        k.src_fx = fd[0]; k.src_fy = fd[1]; k.src_fz = fd[2];
    }
}

// ---------------------------------------------------------------------------------------------
// Session: one prepared simulation on one device.
// ---------------------------------------------------------------------------------------------
struct Session {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    KParams kp{};
    bool reflect = false, savedet = false, use64 = false;
    int block = 256, grid = 0, sms = 0;
    size_t smem = 0;
    size_t nvox = 0, fieldlen = 0;
    int totalgates = 1;
    DevBuf labels, field, shadow, field64, outbuf, detp, detcount, energy, counters, work, err, detpos, pattern;
    DevBuf phase_tab, angle_tab;   // user phase function and launch-angle inverse CDFs
    DevBuf extra_src;              // extra sources, 5 float4 each
    DevBuf replay_seed, replay_w, replay_tof, replay_detid, seeddata, voxwords, voxwords2, traj, trajcount, smat;
    unsigned blocks = 1;       // field blocks of maxgate gates: sources kept apart x detectors of an all-detector replay
    unsigned det_blocks = 1;   // the detector blocks within one source's block
    unsigned halves = 1;       // 2: RF replay, real then imaginary part
    unsigned chans = 1;        // photon sharing: one channel per pattern, adjacent per voxel and gate
    double kernel_ms = 0.0;
    int launches = 0;
    // MCX per-thread seeding: stream count, host/device seed words and the glibc random_r state
    // continuing across runs as MCX's rand() sequence does across respins
    unsigned mcx_streams = 0;
    DevBuf words;
    std::vector<uint32_t> hwords;
    random_data rstate{};
    char rbuf[128];
    long long rseed = -1;

    ~Session() {
        labels.release(); field.release(); shadow.release(); field64.release(); outbuf.release(); detp.release();
        words.release();
        detcount.release(); energy.release(); counters.release(); work.release(); err.release(); detpos.release();
        pattern.release(); phase_tab.release(); angle_tab.release(); extra_src.release(); replay_seed.release(); replay_w.release(); replay_tof.release(); replay_detid.release();
        seeddata.release(); voxwords.release(); voxwords2.release(); traj.release(); trajcount.release(); smat.release();
        // every buffer above is freed on `stream`, which must outlive them
        if (stream) cudaStreamSynchronize(stream);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    void create(const Config* cfg, int dev, bool fp64_field, int gate_cap = 0) {
        device = dev;
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        CK(cudaEventCreate(&ev0));
        CK(cudaEventCreate(&ev1));
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;   // keep freed blocks for the next run instead of returning them
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaDeviceProp prop;
        CK(cudaGetDeviceProperties(&prop, device));
        sms = prop.multiProcessorCount;

        if (cfg->medianum < 1 || cfg->medianum > (unsigned)kMaxMedia)
            MCXG_RAISE(-6, "the GB300 engine supports 1 to 128 media labels");
        if (!cfg->vol) MCXG_RAISE(-4, "the 'vol' field in the input structure can not be empty");
        if (cfg->dim.x >= 32768 || cfg->dim.y >= 32768 || cfg->dim.z >= 32768)
            MCXG_RAISE(-6, "volume dimensions must be below 32768");
        nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        use64 = fp64_field;

        // gates held on the device at once (src/mcx_core.cu:2898-2902, 2944-2956)
        totalgates = (int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5f);
        if (totalgates < 1) totalgates = 1;
        int maxgate = (cfg->maxgate > 0) ? std::min<int>((int)cfg->maxgate, totalgates) : totalgates;
        size_t freeb = 0, totalb = 0;
        cudaMemGetInfo(&freeb, &totalb);
        chans = share_channels(cfg);
        const size_t per_gate = (nvox * (use64 ? sizeof(double) : 2 * sizeof(float)) + nvox * sizeof(float)) * chans;
        const size_t budget = freeb > (size_t)(1u << 30) ? freeb - (size_t)(1u << 30) : freeb / 2;
        if ((size_t)maxgate * per_gate > budget) maxgate = std::max<int>(1, (int)(budget / per_gate));
        if (gate_cap > 0) maxgate = std::min(maxgate, gate_cap);
        // a replay of every detector at once keeps one block of gates per detector
        // (src/mcx_core.cu:2907-2913)
        det_blocks = (cfg->seed == kSEED_FROM_FILE && cfg->replaydet == -1) ? std::max(1u, cfg->detnum) : 1;
        // every source kept apart (srcid -1): one such block per source (src/mcx_core.cu:3039-3046)
        blocks = det_blocks * ((cfg->extrasrclen && cfg->srcid < 0) ? cfg->extrasrclen + 1 : 1);
        // RF replay outputs carry a real and an imaginary field (src/mcx_core.cu:2908-2913)
        halves = (cfg->outputtype == otRF || cfg->outputtype == otRFmus) ? 2 : 1;
        if ((size_t)maxgate * blocks * halves * per_gate > budget)
            maxgate = std::max<int>(1, (int)(budget / (per_gate * blocks * halves)));
        fieldlen = nvox * (size_t)maxgate * blocks * halves * chans;

        // labels: upload the uint32 volume, pack to one byte per voxel on the device; the
        // per-voxel media formats keep MCX's 32-bit words
        const bool words_mode = media_words(cfg->mediabyte);
        if (words_mode) {
            voxwords.alloc(nvox * sizeof(uint32_t), stream);
            err.alloc(sizeof(unsigned), stream);
            CK(cudaMemcpyAsync(voxwords.p, cfg->vol, nvox * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
            if (cfg->mediabyte == kMediaAsgnF2H || cfg->mediabyte == kMedia2LabelSplit) {
                // the second word of every voxel follows the first nvox
                voxwords2.alloc(nvox * sizeof(uint32_t), stream);
                CK(cudaMemcpyAsync(voxwords2.p, cfg->vol + nvox, nvox * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
            }
        } else {
            DevBuf vol32;
            vol32.alloc(nvox * sizeof(uint32_t), stream);
            CK(cudaMemcpyAsync(vol32.p, cfg->vol, nvox * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
            labels.alloc(nvox, stream);
            err.alloc(sizeof(unsigned), stream);
            CK(cudaMemsetAsync(err.p, 0, sizeof(unsigned), stream));
            CK(launch_labels_from_vol(vol32.as<uint32_t>(), labels.as<uint8_t>(), nvox, cfg->medianum, err.as<unsigned>(), stream));
            unsigned e = 0;
            CK(cudaMemcpyAsync(&e, err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            if (e & kErrBadLabel) MCXG_RAISE(-4, "input media optical properties are less than the labels in the volume");
        }

        KParams& k = kp;
        std::memset(&k, 0, sizeof(k));
        k.mediaformat = cfg->mediabyte;
        k.words = voxwords.as<uint32_t>();
        k.words2 = voxwords2.as<uint32_t>();
        k.nx = (int)cfg->dim.x; k.ny = (int)cfg->dim.y; k.nz = (int)cfg->dim.z;
        k.dimxy = cfg->dim.x * cfg->dim.y;
        k.nvox = (unsigned)nvox;
        k.medianum = (int)cfg->medianum;
        for (unsigned i = 0; i < cfg->medianum; i++)
            k.prop[i] = make_float4(cfg->prop[i].mua, cfg->prop[i].mus, cfg->prop[i].g, cfg->prop[i].n);
        k.oneoverc0 = kR_C0 * cfg->unitinmm;
        k.Rtstep = 1.f / cfg->tstep;
        k.maxgate = maxgate;
        k.doreflect = cfg->isreflect ? 1 : 0;
        k.save2pt = cfg->issave2pt ? 1 : 0;
        k.saveref = cfg->issave2pt ? (int)cfg->issaveref : 0;
        k.outputtype = cfg->outputtype;
        k.minenergy = cfg->minenergy;
        k.gscatter = (float)cfg->gscatter;
        k.maxvoidstep = (float)cfg->maxvoidstep;
        std::memcpy(k.bc, cfg->bc, 12);
        reflect = cfg->isreflect != 0;
        for (int i = 0; i < 6; i++)
            if (cfg->bc[i] == BC_REFLECT || cfg->bc[i] == BC_MIRROR) reflect = true;

        // detectors and record layout (src/mcx_core.cu:2840-2847)
        savedet = cfg->issavedet && (cfg->detnum > 0 || std::any_of(cfg->bc + 6, cfg->bc + 12, [](char c) { return c != 0; }));
        const unsigned f = cfg->savedetflag;
        k.savedetflag = f;
        k.nmedia_det = (int)cfg->medianum - 1;
        k.partialdata = (cfg->medianum - 1) * (((f >> 1) & 1u) + ((f >> 2) & 1u) + ((f >> 3) & 1u));
        k.reclen = k.partialdata + (f & 1u) + 3u * (((f >> 4) & 1u) + ((f >> 5) & 1u)) + ((f >> 6) & 1u) +
                   (cfg->polmedianum ? 4u * ((f >> 7) & 1u) : 0u);
        k.maxdet = cfg->maxdetphoton;
        k.ndet = (int)cfg->detnum;
        if (cfg->detnum) {
            detpos.alloc(sizeof(float4) * cfg->detnum, stream);
            CK(cudaMemcpyAsync(detpos.p, cfg->detpos, sizeof(float4) * cfg->detnum, cudaMemcpyHostToDevice, stream));
            k.detpos = detpos.as<float4>();
        }

        // source: pattern intensities on the device, launch state
        const size_t npat = source_pattern_len(cfg);
        if (npat) {
            pattern.alloc(npat * sizeof(float), stream);
            CK(cudaMemcpyAsync(pattern.p, cfg->srcpattern, npat * sizeof(float), cudaMemcpyHostToDevice, stream));
        }
        fill_source(k, cfg, pattern.as<float>());
        // user phase function and launch-angle tables (src/mcx_core.cu:1804-1836 stage them in
        // shared memory; here they are read through the read-only cache)
        k.nextra = (int)cfg->extrasrclen;
        k.srcid = cfg->srcid;
        if (k.nextra) {
            // position (weight 1 when 0), unit direction, param1, param2, and the focal length
            // classified on the host as for the primary source (src/mcx_utils.c:1688-1692)
            std::vector<float4> xs;
            for (unsigned i = 0; i < cfg->extrasrclen; i++) {
                const ExtraSrc& e = cfg->srcdata[i];
                float4 p = e.srcpos;
                if (p.w == 0.f) p.w = 1.f;
                float3 v = f3(e.srcdir.x, e.srcdir.y, e.srcdir.z);
                const float n = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
                if (n > 0.f) { v.x /= n; v.y /= n; v.z /= n; }
                const float f = e.srcdir.w;
                const int focus = std::isnan(f) ? kFocusIsotropic : std::isinf(f) ? kFocusLambertian
                                : (f != 0.f) ? kFocusLength : kFocusNone;
                xs.push_back(p);
                xs.push_back(make_float4(v.x, v.y, v.z, 0.f));
                xs.push_back(e.srcparam1);
                xs.push_back(e.srcparam2);
                xs.push_back(make_float4((float)focus, std::isfinite(f) ? f : 0.f, 0.f, 0.f));
            }
            extra_src.alloc(xs.size() * sizeof(float4), stream);
            CK(cudaMemcpyAsync(extra_src.p, xs.data(), xs.size() * sizeof(float4), cudaMemcpyHostToDevice, stream));
            CK(cudaStreamSynchronize(stream));
            k.extrasrc = extra_src.as<float4>();
        }
        k.nphase = (cfg->nphase > 2) ? (int)cfg->nphase : 0;
        k.nangle = (int)cfg->nangle;
        if (k.nphase) {
            phase_tab.alloc(k.nphase * sizeof(float), stream);
            CK(cudaMemcpyAsync(phase_tab.p, cfg->invcdf, k.nphase * sizeof(float), cudaMemcpyHostToDevice, stream));
            k.invcdf = phase_tab.as<float>();
        }
        if (k.nangle) {
            angle_tab.alloc(k.nangle * sizeof(float), stream);
            CK(cudaMemcpyAsync(angle_tab.p, cfg->angleinvcdf, k.nangle * sizeof(float), cudaMemcpyHostToDevice, stream));
            k.angleinvcdf = angle_tab.as<float>();
        }
        {
            std::lock_guard<std::mutex> g(g_override_mu);
            k.step_cap = g_step_cap;      // a photon longer than this is a fault: flagged and stopped
        }

        // photon replay (MCX's SEED_FROM_FILE, prepared by mcx_replayinit) and seed saving
        k.replay = (cfg->seed == kSEED_FROM_FILE) ? 1 : 0;
        k.replaydet = cfg->replaydet;
        k.detnum = (int)cfg->detnum;
        k.omega = cfg->omega;
        k.rf_offset = fieldlen / halves;
        if (k.replay) {
            const size_t n = (size_t)cfg->nphoton;
            replay_seed.alloc(n * kSeedBytes, stream);
            replay_w.alloc(n * sizeof(float), stream);
            replay_tof.alloc(n * sizeof(float), stream);
            replay_detid.alloc(n * sizeof(int), stream);
            CK(cudaMemcpyAsync(replay_seed.p, cfg->replay.seed, n * kSeedBytes, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(replay_w.p, cfg->replay.weight, n * sizeof(float), cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(replay_tof.p, cfg->replay.tof, n * sizeof(float), cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(replay_detid.p, cfg->replay.detid, n * sizeof(int), cudaMemcpyHostToDevice, stream));
            k.replay_seed = replay_seed.as<unsigned long long>();
            k.replay_w = replay_w.as<float>();
            k.replay_tof = replay_tof.as<float>();
            k.replay_detid = replay_detid.as<int>();
        }
        k.saveseed = (cfg->issaveseed && savedet) ? 1 : 0;

        // output and scratch buffers
        field.alloc(fieldlen * sizeof(float), stream);
        outbuf.alloc(fieldlen * sizeof(float), stream);
        if (use64) field64.alloc(fieldlen * sizeof(double), stream);
        else shadow.alloc(fieldlen * sizeof(float), stream);
        if (savedet) {
            detp.alloc((size_t)k.maxdet * k.reclen * sizeof(float), stream);
            detcount.alloc(sizeof(unsigned), stream);
        }
        if (k.saveseed) {
            seeddata.alloc((size_t)k.maxdet * kSeedBytes, stream);
            k.seeddata = seeddata.as<unsigned long long>();
        }
        if (cfg->polmedianum) {
            // polarised media: the Mueller tables of every medium after the background
            const size_t n = (size_t)cfg->polmedianum * kNAngles;
            smat.alloc(n * sizeof(float4), stream);
            CK(cudaMemcpyAsync(smat.p, cfg->smatrix, n * sizeof(float4), cudaMemcpyHostToDevice, stream));
            k.polarized = 1;
            k.smatrix = smat.as<float4>();
            k.srciquv = cfg->srciquv;
        }
        if (cfg->debuglevel & (kDebugMove | kDebugMoveOnly)) {
            // trajectory records (src/mcx_core.cu:3158-3160): maxjumpdebug x 6 floats
            k.traj_max = cfg->maxjumpdebug;
            k.traj_reclen = (int)(kTrajRecLen + (cfg->istrajstokes ? 4u : 0u));
            traj.alloc((size_t)std::max(1u, k.traj_max) * k.traj_reclen * sizeof(float), stream);
            trajcount.alloc(sizeof(unsigned), stream);
            k.traj = traj.as<float>();
            k.traj_count = trajcount.as<unsigned>();
        }
        energy.alloc(sizeof(double) * kNumEnergy, stream);
        counters.alloc(sizeof(unsigned long long) * kNumCounters, stream);
        work.alloc(sizeof(unsigned long long), stream);
        k.labels = labels.as<uint8_t>();
        k.field = field.as<float>();
        k.shadow = shadow.as<float>();
        k.field64 = field64.as<double>();
        k.detp = detp.as<float>();
        k.detcount = detcount.as<unsigned>();
        k.energy = energy.as<double>();
        k.counters = counters.as<unsigned long long>();
        k.errflag = err.as<unsigned>();
        k.work = work.as<unsigned long long>();
        reset();
        set_window(cfg->tstart, cfg->tstart + cfg->tstep * (float)k.maxgate);   // first gate group

        configure_launch(cfg);

        k.seed_mode = seeding_mode();
        if (k.seed_mode == 1) {
            // the thread count MCX's autopilot picks on this device (src/mcx_core.cu:2554-2608,
            // 2688-2695, 3050-3053), or the user's nthread/nblocksize without autopilot
            const int v = prop.major * 10 + prop.minor;
            const int smxblock = v < 30 ? 8 : (v < 50 ? 16 : 32);
            long long block_ref, threads;
            if (cfg->autopilot) {
                block_ref = std::max(prop.maxThreadsPerMultiProcessor / smxblock, 64);
                threads = block_ref * smxblock * (long long)prop.multiProcessorCount * (v <= 75 ? 1 : 2);
            } else {
                block_ref = std::max(1u, cfg->nblocksize);
                threads = cfg->nthread;
            }
            threads -= threads % block_ref;
            if (threads <= 0) MCXG_RAISE(-6, "invalid thread count for MCX seeding");
            mcx_streams = (unsigned)threads;
            k.mcx_streams = mcx_streams;
            words.alloc((size_t)mcx_streams * 4 * sizeof(uint32_t), stream);
            k.mcx_words = words.as<uint32_t>();
            hwords.resize((size_t)mcx_streams * 4);
        }
    }

    // MCX's seed words for the next run: (rand()<<16)|(rand()<<1)|(rand()>>14), four per thread,
    // continuing the sequence srand(seed) started (src/mcx_core.cu:3247-3251, 3381-3387).
    void mcx_seed_words(uint64_t seed) {
        if ((long long)seed != rseed) {
            std::memset(&rstate, 0, sizeof(rstate));
            initstate_r((unsigned)seed, rbuf, sizeof(rbuf), &rstate);
            rseed = (long long)seed;
        }
        for (auto& wd : hwords) {
            int32_t a, b, c;
            random_r(&rstate, &a);
            random_r(&rstate, &b);
            random_r(&rstate, &c);
            wd = ((uint32_t)a << 16) | ((uint32_t)b << 1) | ((uint32_t)c >> 14);
        }
        CK(cudaMemcpyAsync(words.p, hwords.data(), hwords.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
    }

    // Block size, CTAs per SM and refill chunk; the deposit tile placed over the source.
    void configure_launch(const Config* cfg) {
        LaunchOverride o;
        {
            std::lock_guard<std::mutex> g(g_override_mu);
            o = g_override;
        }
        block = o.block > 0 ? std::min(o.block, 256) : 256;
        // a CTA-per-SM cap of 1-3 selects the larger register budget
        set_transport_variant((o.blocks_per_sm > 0 && o.blocks_per_sm <= 3) ? 3 : 4);
        choose_tile(cfg, o.tile);
        smem = transport_smem_bytes(kp, block, savedet);
        int bps = transport_blocks_per_sm(reflect, savedet, transport_mode(kp), block, smem);
        if (bps <= 0) {
            kp.tile_on = 0;
            smem = transport_smem_bytes(kp, block, savedet);
            bps = transport_blocks_per_sm(reflect, savedet, transport_mode(kp), block, smem);
        }
        if (bps <= 0) MCXG_RAISE(-6, "the transport kernel does not fit on this device");
        if (o.blocks_per_sm > 0) bps = std::min(bps, o.blocks_per_sm);
        grid = bps * sms;
        kp.chunk = o.chunk > 0 ? o.chunk : 64;
    }

    // Deposit tile over the entry point in a shared-memory budget of tile_kb KB (default 16).
    void choose_tile(const Config* cfg, int tile_kb) {
        place_tile(kp, std::max(kMinTileKB, (tile_kb >= 0) ? tile_kb : 16));
        (void)cfg;
    }

    // Configuration signature for the tuning cache: what changes the best launch shape.
    std::string signature() const {
        char buf[256];
        snprintf(buf, sizeof(buf), "%d:%d:%d:%d:%d:%d:%d:%u:%d:%d", kp.nx, kp.ny, kp.nz, kp.maxgate, kp.medianum, (int)reflect,
                 (int)savedet, kp.src_idx, kp.seed_mode, transport_variant());
        return buf;
    }

    // Pick the deposit-tile budget from short pilot launches over {2, 16, 32} KB (cached per
    // signature).  Pilot photons go to the session's buffers, which are cleared afterwards.
    void autotune(uint64_t nphoton) {
        const std::string sig = signature();
        {
            std::lock_guard<std::mutex> g(g_tune_mu);
            for (auto& e : g_tune_cache)
                if (e.first == sig) {
                    apply_tile(e.second);
                    return;
                }
        }
        const uint64_t pilot = std::max<uint64_t>(500000, std::min<uint64_t>(4000000, nphoton / 64));
        int best_kb = 16;
        float best = 1e30f;
        for (int kb : {kMinTileKB, 16, 32}) {
            apply_tile(kb);
            run(0, pilot, 0x5eed);          // first launch of a shape warms it up
            const float ms = run(pilot, pilot, 0x5eed);
            if (ms < best) {
                best = ms;
                best_kb = kb;
            }
        }
        apply_tile(best_kb);
        reset();
        std::lock_guard<std::mutex> g(g_tune_mu);
        g_tune_cache.emplace_back(sig, best_kb);
    }

    void apply_tile(int kb) {
        choose_tile(nullptr, kb);
        smem = transport_smem_bytes(kp, block, savedet);
        int bps = transport_blocks_per_sm(reflect, savedet, transport_mode(kp), block, smem);
        if (bps <= 0) {
            kp.tile_on = 0;
            smem = transport_smem_bytes(kp, block, savedet);
            bps = transport_blocks_per_sm(reflect, savedet, transport_mode(kp), block, smem);
        }
        grid = std::max(1, bps) * sms;
    }

    void reset() {
        CK(cudaMemsetAsync(field.p, 0, field.bytes, stream));
        if (shadow.p) CK(cudaMemsetAsync(shadow.p, 0, shadow.bytes, stream));
        if (field64.p) CK(cudaMemsetAsync(field64.p, 0, field64.bytes, stream));
        if (detcount.p) CK(cudaMemsetAsync(detcount.p, 0, detcount.bytes, stream));
        if (kp.saveref > 1 && detp.p) CK(cudaMemsetAsync(detp.p, 0, detp.bytes, stream));     // per-voxel sums
        CK(cudaMemsetAsync(energy.p, 0, energy.bytes, stream));
        CK(cudaMemsetAsync(counters.p, 0, counters.bytes, stream));
        CK(cudaMemsetAsync(err.p, 0, err.bytes, stream));
        kernel_ms = 0.0;
        launches = 0;
    }

    void set_window(float twin0, float twin1) {
        kp.twin0 = twin0;
        kp.twin1 = twin1;
    }

    // One persistent transport launch over photons [offset, offset + n).
    float run(uint64_t offset, uint64_t n, uint64_t seed) {
        CK(cudaSetDevice(device));
        kp.photon_offset = offset;
        kp.nphoton = n;
        kp.seed = seed;
        if (kp.seed_mode == 1) {
            mcx_seed_words(seed);
            kp.mcx_per = (unsigned)(n / mcx_streams);
            kp.mcx_odd = (unsigned)(n - (uint64_t)kp.mcx_per * mcx_streams);
        }
        CK(cudaMemsetAsync(work.p, 0, sizeof(unsigned long long), stream));
        CK(cudaEventRecord(ev0, stream));
        CK(launch_transport(kp, reflect, savedet, grid, block, smem, stream));
        CK(cudaEventRecord(ev1, stream));
        CK(cudaEventSynchronize(ev1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ev0, ev1));
        kernel_ms += ms;
        launches++;
        return ms;
    }

    // Queue a cleared-buffer launch over photons [offset, offset + n) on stream `s` without
    // waiting (the batch captures these into one graph).  MCX seeding words must be in place.
    // One repetition enqueued on `s` (for graph capture).  `fresh` starts a gate window: field,
    // energies and counters cleared; later repetitions of the window add to them.
    void enqueue(cudaStream_t s, uint64_t offset, uint64_t n, uint64_t seed, bool fresh = true) {
        kp.photon_offset = offset;
        kp.nphoton = n;
        kp.seed = seed;
        if (kp.seed_mode == 1) {
            kp.mcx_per = (unsigned)(n / mcx_streams);
            kp.mcx_odd = (unsigned)(n - (uint64_t)kp.mcx_per * mcx_streams);
        }
        if (fresh) {
            CK(cudaMemsetAsync(field.p, 0, field.bytes, s));
            if (shadow.p) CK(cudaMemsetAsync(shadow.p, 0, shadow.bytes, s));
            if (field64.p) CK(cudaMemsetAsync(field64.p, 0, field64.bytes, s));
            CK(cudaMemsetAsync(energy.p, 0, energy.bytes, s));
            CK(cudaMemsetAsync(counters.p, 0, counters.bytes, s));
            CK(cudaMemsetAsync(err.p, 0, err.bytes, s));
        }
        if (detcount.p) CK(cudaMemsetAsync(detcount.p, 0, detcount.bytes, s));
        if (kp.saveref > 1 && detp.p) CK(cudaMemsetAsync(detp.p, 0, detp.bytes, s));
        if (trajcount.p) CK(cudaMemsetAsync(trajcount.p, 0, trajcount.bytes, s));
        CK(cudaMemsetAsync(work.p, 0, sizeof(unsigned long long), s));
        CK(launch_transport(kp, reflect, savedet, grid, block, smem, s));
        launches = 1;
    }

    // Merge shadow copies and scale into a device buffer of the caller (fieldlen floats), in
    // stream order: nothing crosses to the host.
    void read_field_device(float* dev, float scale, int positive_only) {
        CK(cudaSetDevice(device));
        CK(launch_merge_field(dev, field.as<float>(), shadow.as<float>(), field64.as<double>(), fieldlen, scale,
                              positive_only, stream));
    }

    // Merge shadow copies, optionally scale, and copy the field out.
    void read_field(float* host, float scale, int positive_only) {
        CK(cudaSetDevice(device));
        CK(launch_merge_field(outbuf.as<float>(), field.as<float>(), shadow.as<float>(), field64.as<double>(), fieldlen, scale,
                              positive_only, stream));
        CK(cudaMemcpyAsync(host, outbuf.p, fieldlen * sizeof(float), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
    }

    unsigned detected() {
        if (!detcount.p) return 0;
        if (kp.saveref > 1) return kp.maxdet;      // one record per voxel (src/mcx_core.cu:2520-2522)
        unsigned d = 0;
        CK(cudaMemcpyAsync(&d, detcount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        return d;
    }

    void read_stats(mcxg_stats* st) {
        CK(cudaSetDevice(device));
        double e[kNumEnergy];
        unsigned long long c[kNumCounters];
        unsigned ef = 0;
        CK(cudaMemcpyAsync(e, energy.p, sizeof(e), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(c, counters.p, sizeof(c), cudaMemcpyDeviceToHost, stream));
        CK(cudaMemcpyAsync(&ef, err.p, sizeof(ef), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        st->e_launch = e[kELaunch]; st->e_escape = e[kEEscape]; st->e_detect = e[kEDetect];
        st->e_absdep = e[kEAbsDep]; st->e_absother = e[kEAbsOther];
        st->n_steps = c[kCntSteps]; st->n_scatter = c[kCntScatter]; st->n_deposit = c[kCntDeposit];
        st->n_launch = c[kCntLaunch]; st->n_photon = c[kCntPhoton]; st->n_detected = detected();
        st->n_tile_deposit = c[kCntTileDeposit];
        st->kernel_ms = kernel_ms;
        st->grid = grid; st->block = block; st->chunk = kp.chunk; st->launches = launches;
        st->error_flags = ef;
    }
};

}  // namespace mcxg

using namespace mcxg;

// ---------------------------------------------------------------------------------------------
// Error plumbing
// ---------------------------------------------------------------------------------------------
extern "C" const char* mcxg_last_error(void) { return t_err_msg.c_str(); }
extern "C" int mcxg_last_error_id(void) { return t_err_id; }
extern "C" void mcxg_clear_error(void) { t_err_id = 0; t_err_msg.clear(); }
extern "C" void mcxg_set_error(int id, const char* msg) { t_err_id = id; t_err_msg = msg ? msg : ""; }
extern "C" int mcxg_get_stats(mcxg_stats* out) {
    if (!out) return -1;
    *out = t_stats;
    return 0;
}
extern "C" void mcxg_set_seeding(int mode) {
    std::lock_guard<std::mutex> g(g_override_mu);
    g_seeding = (mode == 1) ? 1 : 0;
}

extern "C" void mcxg_set_field_precision(int bits) {
    std::lock_guard<std::mutex> g(g_override_mu);
    g_field_bits = (bits == 64) ? 64 : 32;
}

extern "C" void mcxg_set_step_cap(unsigned int steps) {
    std::lock_guard<std::mutex> g(g_override_mu);
    g_step_cap = steps ? steps : kDefaultStepCap;
}

extern "C" void mcxg_set_launch(int block, int blocks_per_sm, int chunk, int tile) {
    std::lock_guard<std::mutex> g(g_override_mu);
    g_override.block = block;
    g_override.blocks_per_sm = blocks_per_sm;
    g_override.chunk = chunk;
    g_override.tile = tile;
}

// ---------------------------------------------------------------------------------------------
// mcx_list_gpu (src/mcx_core.cu:2621-2726)
// ---------------------------------------------------------------------------------------------
extern "C" int mcx_list_gpu(Config* cfg, GPUInfo** info) {
    try {
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess) {
            if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                MCXG_RAISE(-(int)e, "A CUDA-capable GPU is not found or configured");
            MCXG_RAISE(-(int)e, cudaGetErrorString(e));
        }
        if (count == 0) {
            if (cfg->flog) fprintf(cfg->flog, "ERROR: No CUDA-capable GPU device found\n");
            return 0;
        }
        *info = (GPUInfo*)calloc((size_t)count, sizeof(GPUInfo));
        if (cfg->gpuid && cfg->gpuid > count) {
            if (cfg->flog) fprintf(cfg->flog, "ERROR: Specified GPU ID is out of range\n");
            free(*info);
            *info = nullptr;
            return 0;
        }
        int active = 0;
        for (int dev = 0; dev < count; dev++) {
            cudaDeviceProp dp;
            CK(cudaGetDeviceProperties(&dp, dev));
            if (cfg->isgpuinfo == 3) {
                active++;
            } else if (cfg->deviceid[dev] == '1') {
                cfg->deviceid[dev] = '\0';
                cfg->deviceid[active] = (char)(dev + 1);
                active++;
            }
            GPUInfo& g = (*info)[dev];
            strncpy(g.name, dp.name, MCXG_SESSION_LEN - 1);
            g.id = dev + 1;
            g.devcount = count;
            g.major = dp.major;
            g.minor = dp.minor;
            g.globalmem = dp.totalGlobalMem;
            g.constmem = dp.totalConstMem;
            g.sharedmem = dp.sharedMemPerBlock;
            g.regcount = dp.regsPerBlock;
            int clk = 0;
            cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
            g.clock = clk;
            g.sm = dp.multiProcessorCount;
            g.core = dp.multiProcessorCount * 128;
            g.maxmpthread = dp.maxThreadsPerMultiProcessor;
            g.maxgate = cfg->maxgate;
            // this engine's persistent launch: 256-thread CTAs filling every SM
            g.autoblock = 256;
            g.autothread = g.autoblock * (dp.maxThreadsPerMultiProcessor / g.autoblock) * g.sm;
            if (cfg->isgpuinfo) {
                FILE* o = stdout;
                fprintf(o, "=============================   GPU Information  ================================\n");
                fprintf(o, "Device %d of %d:\t\t%s\n", g.id, g.devcount, g.name);
                fprintf(o, "Compute Capability:\t%u.%u\n", g.major, g.minor);
                fprintf(o, "Global Memory:\t\t%.0f B\nConstant Memory:\t%.0f B\nShared Memory:\t\t%.0f B\nRegisters:\t\t%u\nClock Speed:\t\t%.2f GHz\n",
                        (double)g.globalmem, (double)g.constmem, (double)g.sharedmem, (unsigned)g.regcount, g.clock * 1e-6f);
                fprintf(o, "Number of SMs:\t\t%u\nNumber of Cores:\t%u\n", g.sm, g.core);
                fprintf(o, "Auto-thread:\t\t%d\nAuto-block:\t\t%d\n", g.autothread, g.autoblock);
            }
        }
        if (cfg->isgpuinfo == 2 && cfg->parentid == mpStandalone) exit(0);
        if (active < MCXG_MAX_DEVICE) cfg->deviceid[active] = '\0';
        return active;
    } catch (const Error& e) {
        report(e);
        return 0;
    }
}

// ---------------------------------------------------------------------------------------------
// mcx_run_simulation (src/mcx_core.cu:2740-4110)
// ---------------------------------------------------------------------------------------------
namespace {

// Settings every run path rejects (MCX error ids).
void check_config(const Config* cfg) {
    if (cfg->seed == kSEED_FROM_FILE &&
        !(cfg->replay.seed && cfg->replay.weight && cfg->replay.tof && cfg->replay.detid))
        MCXG_RAISE(-6, "a replay needs the detected photons' seeds, weights, times of flight and detector ids (mcx_replayinit)");
    const int ot = cfg->outputtype;
    if ((ot == otJacobian || ot == otWP || ot == otDCS || ot == otRF || ot == otRFmus || ot == otWLTOF || ot == otWPTOF) &&
        cfg->seed != kSEED_FROM_FILE)
        MCXG_RAISE(-6, "the Jacobian and scattering-count outputs need a replay run (seed from the detected photons)");
    if (ot < otFlux || ot > otWPTOF) MCXG_RAISE(-6, "unknown output type");
    if (cfg->respin == 0) MCXG_RAISE(-1, "respin number can not be 0, check your -r/--repeat input or cfg.respin value");
    if (cfg->mediabyte > 4 && !media_words(cfg->mediabyte))
        MCXG_RAISE(-6, "the GB300 engine supports label media (mediabyte 1, 2, 4) and the per-voxel formats 96-104");
    if ((cfg->mediabyte == kMediaAsF2H || cfg->mediabyte == kMediaMuaFloat || cfg->mediabyte == kMediaAsHalf) && cfg->medianum < 2)
        MCXG_RAISE(-4, "the per-voxel media format needs the 2nd row of prop for the properties it does not store");
    if ((cfg->mediabyte == kMediaAsgnByte || cfg->mediabyte == kMediaAsShort) && cfg->medianum < 3)
        MCXG_RAISE(-4, "the interpolating media formats need prop rows 2 and 3 as their end points");
    if (cfg->mediabyte == kMedia2LabelSplit && cfg->vol) {
        // both labels of every split voxel index the property table
        const size_t nv = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        for (size_t i = 0; i < nv; i++)
            if (((cfg->vol[i] & kMED_MASK) >> 24) >= cfg->medianum || ((cfg->vol[i] >> 16) & 0xFFu) >= cfg->medianum)
                MCXG_RAISE(-6, "a split voxel's label exceeds the number of media");
    }
    if (cfg->mediabyte == kMedia2LabelMix && cfg->vol) {
        // both tissue labels of every word index the property table
        const size_t nv = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        for (size_t i = 0; i < nv; i++)
            if ((cfg->vol[i] & 0xFFu) >= cfg->medianum || ((cfg->vol[i] >> 8) & 0xFFu) >= cfg->medianum)
                MCXG_RAISE(-6, "a MEDIA_2LABEL_MIX voxel's label exceeds the number of media");
    }
    if (cfg->mediabyte == kMediaLabelHalf && cfg->vol) {
        // the word's 14-bit label indexes the property table
        const size_t nv = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
        for (size_t i = 0; i < nv; i++)
            if ((cfg->vol[i] & 0x3FFFu) >= cfg->medianum)
                MCXG_RAISE(-6, "a MEDIA_LABEL_HALF voxel's label exceeds the number of media");
    }
    if (cfg->polmedianum && (cfg->mediabyte > 4 || !cfg->smatrix || cfg->medianum != cfg->polmedianum + 1))
        MCXG_RAISE(-6, "polarized media need label volumes and the Mueller tables of mcx_prep_polarized");
    check_source(cfg);
}

// Output buffers and counters of a run, as mcx_run_simulation leaves them before its first
// launch (src/mcx_core.cu:2907-2921): exportfield is accumulated into, exportdetected grows.
void begin_outputs(Config* cfg, const Session& S, bool host_field = true) {
    if (host_field && cfg->exportfield == nullptr && cfg->issave2pt) cfg->exportfield = (float*)calloc(S.fieldlen, sizeof(float));
    if (cfg->exportdetected == nullptr)
        cfg->exportdetected = (float*)malloc((size_t)S.kp.reclen * std::max(1u, cfg->maxdetphoton) * sizeof(float));
    if (S.kp.saveseed && cfg->seeddata == nullptr)
        cfg->seeddata = malloc((size_t)std::max(1u, cfg->maxdetphoton) * kSeedBytes);
    cfg->his.seedbyte = S.kp.saveseed ? (unsigned)kSeedBytes : 0u;
    cfg->detectedcount = 0;
    cfg->his.detected = 0;
    cfg->his.respin = cfg->respin;
    cfg->his.colcount = S.kp.reclen;
    cfg->energytot = 0.0;
    cfg->energyabs = 0.0;
    cfg->energyesc = 0.0;
    cfg->runtime = 0;
    if (S.totalgates > S.kp.maxgate && cfg->isnormalized) {
        if (cfg->flog)
            fprintf(cfg->flog, "WARNING: GPU memory can not hold all time gates, disabling normalization to allow multiple runs\n");
        cfg->isnormalized = 0;
    }
}

// Detected photons of the last launch appended to exportdetected (src/mcx_core.cu:3645-3666).
void append_detected(Config* cfg, Session& S, std::mutex* mu = nullptr) {
    if (!S.savedet) return;
    const unsigned reclen = S.kp.reclen;
    const unsigned det = S.detected();
    std::unique_lock<std::mutex> lk;
    if (mu) lk = std::unique_lock<std::mutex>(*mu);
    cfg->his.detected += det;
    const unsigned keep = std::min(det, cfg->maxdetphoton);
    if (det > cfg->maxdetphoton && cfg->flog)
        fprintf(cfg->flog, "WARNING: the detected photon number is more than what your have specified (%u > %u), please use the -H option to specify a greater number\n",
                det, cfg->maxdetphoton);
    if (keep && cfg->exportdetected) {
        cfg->exportdetected = (float*)realloc(cfg->exportdetected, (cfg->detectedcount + keep) * (size_t)reclen * sizeof(float));
        CK(cudaMemcpyAsync(cfg->exportdetected + cfg->detectedcount * reclen, S.detp.p, (size_t)keep * reclen * sizeof(float),
                           cudaMemcpyDeviceToHost, S.stream));
        if (S.kp.saveseed && cfg->seeddata) {      // the seeds of the same photons (src/mcx_core.cu:3628-3655)
            cfg->seeddata = realloc(cfg->seeddata, (cfg->detectedcount + keep) * kSeedBytes);
            CK(cudaMemcpyAsync((char*)cfg->seeddata + cfg->detectedcount * kSeedBytes, S.seeddata.p, (size_t)keep * kSeedBytes,
                               cudaMemcpyDeviceToHost, S.stream));
        }
        CK(cudaStreamSynchronize(S.stream));
        cfg->detectedcount += keep;
    }
}

// Trajectory records of the last launch appended to exportdebugdata (src/mcx_core.cu:3594-3614).
void append_trajectory(Config* cfg, Session& S, std::mutex* mu = nullptr) {
    if (!S.kp.traj) return;
    unsigned rec = 0;
    CK(cudaMemcpyAsync(&rec, S.trajcount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, S.stream));
    CK(cudaStreamSynchronize(S.stream));
    std::unique_lock<std::mutex> lk;
    if (mu) lk = std::unique_lock<std::mutex>(*mu);
    if (rec > S.kp.traj_max && cfg->flog)
        fprintf(cfg->flog, "WARNING: the saved trajectory positions are more than what your have specified (%u > %u), please use the --maxjumpdebug option to specify a greater number\n",
                rec, S.kp.traj_max);
    else if (rec && cfg->flog)
        fprintf(cfg->flog, "saved trajectory positions: %u, total: %u\t", rec, cfg->debugdatalen + rec);
    rec = std::min(rec, S.kp.traj_max);
    if (rec) {
        cfg->exportdebugdata = (float*)realloc(cfg->exportdebugdata,
                                               ((size_t)cfg->debugdatalen + rec) * S.kp.traj_reclen * sizeof(float));
        if (!cfg->exportdebugdata) MCXG_RAISE(-4, "out of host memory for the trajectory records");
        CK(cudaMemcpyAsync(cfg->exportdebugdata + (size_t)cfg->debugdatalen * S.kp.traj_reclen, S.traj.p,
                           (size_t)rec * S.kp.traj_reclen * sizeof(float), cudaMemcpyDeviceToHost, S.stream));
        CK(cudaStreamSynchronize(S.stream));
        cfg->debugdatalen += rec;
    }
}

// End of one gate window: statistics, energies, normalised field added to exportfield
// (src/mcx_core.cu:3716-3770, 3823-3925).
// With several devices (src/mcx_core.cu:3730-3759) their energies are summed first, so one
// normaliser scales every device's field, and the scaled fields are summed into exportfield.
void finish_window(Config* cfg, const std::vector<Session*>& SS, std::vector<float>& host_field, mcxg_stats& total,
                   float* dev_out = nullptr) {
    double e_launch = 0.0;
    for (Session* D : SS) {
        mcxg_stats st{};
        D->read_stats(&st);
        if (st.error_flags & kErrStepCap)
            MCXG_RAISE(-6, "a photon exceeded the per-photon step cap; the simulation was stopped");
        if (st.error_flags & kErrIndex)
            MCXG_RAISE(-6, "internal error: a photon's voxel index left the volume; the photon was stopped");
        total.e_launch += st.e_launch; total.e_escape += st.e_escape; total.e_detect += st.e_detect;
        total.e_absdep += st.e_absdep; total.e_absother += st.e_absother;
        total.n_steps += st.n_steps; total.n_scatter += st.n_scatter; total.n_deposit += st.n_deposit;
        total.n_launch += st.n_launch; total.n_photon += st.n_photon; total.n_detected += st.n_detected;
        total.n_tile_deposit += st.n_tile_deposit;
        total.grid = st.grid; total.block = st.block; total.chunk = st.chunk; total.launches += st.launches;
        total.error_flags |= st.error_flags;
        cfg->energytot += st.e_launch;
        cfg->energyesc += st.e_escape + st.e_detect;
        e_launch += st.e_launch;
    }
    Session& S = *SS[0];

    if (cfg->issave2pt) {
        // normalisation (src/mcx_core.cu:3823-3925): flux scale = unitinmm/(Etot*Vvox*tstep)
        float scale = 1.f;
        std::vector<float> block_scale;         // all-detector replay: one scale per detector block
        std::vector<float> chan_scale;          // photon sharing: one scale per pattern
        const int ot = cfg->outputtype;
        const bool path_units = (ot == otJacobian || ot == otRF || ot == otWLTOF);
        if (cfg->isnormalized && e_launch > 0.0) {
            const double Vvox = (double)cfg->steps.x * cfg->steps.y * cfg->steps.z;
            if (ot == otFlux || ot == otFluence) {
                double sc = cfg->unitinmm / (cfg->energytot * Vvox * cfg->tstep);
                if (ot == otFluence) sc *= cfg->tstep;
                scale = (float)sc;
            } else if (ot == otEnergy || ot == otL) {
                scale = (float)(1.0 / cfg->energytot);
            } else if (cfg->seed == kSEED_FROM_FILE && cfg->replaydet == -1) {
                // each detector's block over its replayed weight; paths carry unitinmm.  MCX scales
                // the detector blocks of the first source only (src/mcx_core.cu:3845-3873): with
                // every source kept apart, the other sources' blocks stay as accumulated
                for (unsigned d = 1; d <= S.det_blocks; d++) {
                    float sd = path_units ? cfg->unitinmm : 1.f;
                    if (cfg->isnormalized != 2) {
                        double sum = 0.0;
                        for (size_t i = 0; i < (size_t)cfg->nphoton; i++)
                            if ((unsigned)(cfg->replay.detid[i] & 0xFFFF) == d) sum += cfg->replay.weight[i];
                        sd = (sum > 0.0) ? (float)((path_units ? cfg->unitinmm : 1.0) / sum) : 0.f;
                    }
                    block_scale.push_back(sd);
                }
                scale = block_scale.empty() ? 1.f : block_scale.back();
            } else {
                double sum = 0.0;
                for (size_t i = 0; i < (size_t)cfg->nphoton; i++) sum += cfg->replay.weight[i];
                scale = (sum > 0.0) ? (float)(cfg->unitinmm / sum) : 0.f;
            }
            // every source simulated apart: each got 1/(n+1) of the photons (3908-3910); in an
            // all-detector replay this reaches the reported normaliser only, as in MCX
            if (cfg->extrasrclen && cfg->srcid < 0) scale *= (float)(cfg->extrasrclen + 1);
            if (S.chans > 1) {
                // photon sharing: each pattern's channel over its total intensity
                // (src/mcx_core.cu:3778-3795, 3895-3906), Kahan-summed in float as MCX sums it
                const bool p3 = (unsigned char)cfg->srctype == kSrcPattern3D;
                const int psize = p3 ? (int)cfg->srcparam1.x * (int)cfg->srcparam1.y * (int)cfg->srcparam1.z
                                     : (int)cfg->srcparam1.w * (int)cfg->srcparam2.w;
                for (unsigned c = 0; c < S.chans; c++) {
                    float sum = 0.f, comp = 0.f;
                    for (int p = 0; p < psize; p++) {
                        const float y = cfg->srcpattern[(size_t)p * S.chans + c] - comp;
                        const float t = sum + y;
                        comp = (t - sum) - y;
                        sum = t;
                    }
                    chan_scale.push_back(psize / sum * scale);
                }
                scale = chan_scale[0];
            }
            cfg->normalizer = scale;
            cfg->his.normalizer = scale;
        }
        if (dev_out) {
            if (SS.size() != 1 || !block_scale.empty() || !chan_scale.empty())
                MCXG_RAISE(-4, "a field on the device is given for one device, one pattern and no detector blocks only");
            S.read_field_device(dev_out, scale, cfg->isnormalized == 2);
            return;
        }
        host_field.resize(S.fieldlen);
        for (Session* D : SS) {
        D->read_field(host_field.data(), (block_scale.empty() && chan_scale.empty()) ? scale : 1.f, cfg->isnormalized == 2);
        float* out = cfg->exportfield;
        if (!chan_scale.empty()) {
            for (size_t i = 0; i < S.fieldlen; i++) {
                const float v = host_field[i];
                out[i] += (cfg->isnormalized == 2 && v < 0.f) ? v : v * chan_scale[i % S.chans];
            }
        } else if (block_scale.empty()) {
            for (size_t i = 0; i < S.fieldlen; i++) out[i] += host_field[i];
        } else {
            const size_t per = S.fieldlen / (S.blocks * S.halves);     // one detector's gates
            for (size_t i = 0; i < S.fieldlen; i++) {
                const float v = host_field[i];
                const size_t b = (i / per) % S.blocks;
                out[i] += (cfg->isnormalized == 2 && v < 0.f) ? v : v * (b < S.det_blocks ? block_scale[b] : 1.f);
            }
        }
        }
    }
}

// End of a run: runtime, absorbed energy, the log lines and the standalone file output
// (src/mcx_core.cu:3932-4030).
void end_outputs(Config* cfg, Session& S, double kernel_ms, int reps, int threads = 0) {
    if (threads <= 0) threads = S.grid * S.block;
    cfg->runtime = (unsigned)std::ceil(kernel_ms);
    cfg->energyabs = cfg->energytot - cfg->energyesc;
    // the run summary is printed whatever printnum says: MCX's CLI sets printnum to -1 unless
    // -l is given, and still prints the summary to stdout (src/mcx_core.cu:3996-4030)
    if (cfg->flog) {
        const double np = (double)cfg->nphoton * (cfg->respin > 1 ? cfg->respin : 1);
        if (S.savedet) fprintf(cfg->flog, "detected %u photons, total: %lu\n", cfg->his.detected, (unsigned long)cfg->detectedcount);
        fprintf(cfg->flog, "kernel complete:  \t%.3f ms\n", kernel_ms);
        fprintf(cfg->flog, "simulated %.0f photons (%.0f) with %d threads (repeat x%d)\nMCX simulation speed: %.2f photon/ms\n",
                np, np, threads, reps, np / std::max(1e-3, kernel_ms));
        fprintf(cfg->flog, "total simulated energy: %.2f\tabsorbed: %5.5f%%\n(loss due to initial specular reflection is excluded in the total)\n",
                cfg->energytot, cfg->energytot > 0 ? (cfg->energytot - cfg->energyesc) / cfg->energytot * 100.0 : 0.0);
        fflush(cfg->flog);
    }
    // file output in the standalone CLI (src/mcx_core.cu:3932-3978) when its writers are linked
    if (cfg->parentid == mpStandalone) {
        // (no host field when mcxg_run_batch_device kept it on the device)
        if (cfg->issave2pt && cfg->exportfield && mcx_savedata) mcx_savedata(cfg->exportfield, S.fieldlen, cfg);
        if (cfg->issavedet && cfg->exportdetected && mcx_savedetphoton) {
            cfg->his.unitinmm = cfg->unitinmm;
            cfg->his.savedphoton = (unsigned)cfg->detectedcount;
            cfg->his.totalphoton = (unsigned)cfg->nphoton;
            cfg->his.detected = (unsigned)cfg->detectedcount;
            mcx_savedetphoton(cfg->exportdetected, cfg->seeddata, (int)cfg->detectedcount, 0, cfg);
        }
        // trajectories go through the same writer with their own record length (3980-3987)
        if ((cfg->debuglevel & (kDebugMove | kDebugMoveOnly)) && cfg->exportdebugdata && mcx_savedetphoton) {
            cfg->his.colcount = (unsigned)S.kp.traj_reclen;
            cfg->his.savedphoton = cfg->debugdatalen;
            cfg->his.totalphoton = (unsigned)cfg->nphoton;
            cfg->his.detected = 0;
            mcx_savedetphoton(cfg->exportdebugdata, nullptr, (int)cfg->debugdatalen, 0, cfg);
        }
    }
}

// MCX's -D R (src/mcx_core.cu:3055-3112): instead of a simulation, one GPU thread fills the
// field with the generator's uniforms from four seed words drawn with the C library's rand()
// as MCX draws them; the field is exported and saved like a fluence.
void rng_debug_output(Config* cfg, int gpuid) {
    CK(cudaSetDevice(gpuid));
    const size_t nvox = (size_t)cfg->dim.x * cfg->dim.y * cfg->dim.z;
    int totalgates = (int)((cfg->tend - cfg->tstart) / cfg->tstep + 0.5f);
    if (totalgates < 1) totalgates = 1;
    const int maxgate = (cfg->maxgate > 0) ? std::min<int>((int)cfg->maxgate, totalgates) : totalgates;
    const size_t fieldlen = nvox * (size_t)maxgate;
    if (fieldlen > (size_t)INT32_MAX) MCXG_RAISE(-6, "the -D R field is too large");
    uint32_t words[4];
    for (auto& wd : words) {
        const uint32_t a = (uint32_t)rand(), b = (uint32_t)rand(), c = (uint32_t)rand();
        wd = (a << 16) | (b << 1) | (c >> 14);
    }
    if (cfg->flog) {
        fprintf(cfg->flog, "generating %lu random numbers ... \t", (unsigned long)fieldlen);
        fflush(cfg->flog);
    }
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    DevBuf seeds, out;
    try {
        seeds.alloc(sizeof(words), st);
        out.alloc(fieldlen * sizeof(float), st);
        CK(cudaMemcpyAsync(seeds.p, words, sizeof(words), cudaMemcpyHostToDevice, st));
        CK(launch_rng_test(seeds.as<uint32_t>(), out.as<float>(), (int)fieldlen, st));
        std::vector<float> host(fieldlen);
        CK(cudaMemcpyAsync(host.data(), out.p, fieldlen * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        seeds.release();
        out.release();
        CK(cudaStreamSynchronize(st));
        cudaStreamDestroy(st);
        st = nullptr;
        if (cfg->flog) fprintf(cfg->flog, "kernel complete\n");
        if (cfg->exportfield == nullptr && cfg->issave2pt) cfg->exportfield = (float*)calloc(fieldlen, sizeof(float));
        if (cfg->exportfield) std::memcpy(cfg->exportfield, host.data(), fieldlen * sizeof(float));
        if (cfg->issave2pt && cfg->parentid == mpStandalone && mcx_savedata) mcx_savedata(host.data(), fieldlen, cfg);
    } catch (...) {
        seeds.release();
        out.release();
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
        throw;
    }
}

// Photon shares of the devices listed in cfg->deviceid (src/mcx_core.cu:2980-3007): in
// proportion to cfg->workload, or to the devices' core counts when no workload is given (written
// back to cfg->workload, as MCX's master thread does).  The devices split each launch's photon
// range [0, n) into consecutive pieces; unlike MCX, whose per-device counts are truncated, the
// last device takes the remainder, so the shares always add up to n.
std::vector<double> device_weights(Config* cfg, const GPUInfo* gpu, int ndev) {
    double full = 0.0;
    for (int i = 0; i < ndev; i++) full += cfg->workload[i];
    if (full < kEPS)
        for (int i = 0; i < ndev; i++)
            cfg->workload[i] = gpu ? (float)gpu[cfg->deviceid[i] - 1].core : 1.f;
    std::vector<double> w(ndev);
    for (int i = 0; i < ndev; i++) {
        if (!(cfg->workload[i] > 0.f)) MCXG_RAISE(-1, "workload was unspecified for an active device");
        w[i] = cfg->workload[i];
    }
    return w;
}

void split_photons(const std::vector<double>& w, uint64_t n, std::vector<uint64_t>& offset, std::vector<uint64_t>& count) {
    const size_t nd = w.size();
    double full = 0.0;
    for (double x : w) full += x;
    offset.assign(nd, 0);
    count.assign(nd, 0);
    uint64_t done = 0;
    for (size_t d = 0; d < nd; d++) {
        const uint64_t c = (d + 1 == nd) ? n - done : std::min<uint64_t>(n - done, (uint64_t)((double)n * w[d] / full));
        offset[d] = done;
        count[d] = c;
        done += c;
    }
}

int active_devices(const Config* cfg) {
    int n = 0;
    while (n < MCXG_MAX_DEVICE && cfg->deviceid[n]) n++;
    return n;
}

// Runs f(d) for every device index d, d = 0 on the calling thread and the others on their own
// threads; the first exception (by device order) is rethrown after all have finished.
template <class F>
void on_devices(int ndev, F&& f) {
    if (ndev == 1) {
        f(0);
        return;
    }
    std::vector<std::exception_ptr> err(ndev);
    std::vector<std::thread> th;
    for (int d = 1; d < ndev; d++)
        th.emplace_back([&, d]() {
            try {
                f(d);
            } catch (...) {
                err[d] = std::current_exception();
            }
        });
    try {
        f(0);
    } catch (...) {
        err[0] = std::current_exception();
    }
    for (auto& t : th) t.join();
    for (auto& e : err)
        if (e) std::rethrow_exception(e);
}

// mcx_run_simulation (src/mcx_core.cu:2740-4110).  MCX's front-ends call it once per listed
// device from `#pragma omp parallel`; here the master thread (OpenMP thread 0, or the only caller)
// drives every device of cfg->deviceid from host threads of its own and the other OpenMP
// threads return at once, so the call needs no barrier with the caller's threads.  Each device
// runs its share of every launch on its own session; fields, energies, detected photons and
// trajectories are merged as MCX merges them (3645-3666, 3716-3770), and the one normalisation
// uses the energy of all devices.  The same device may be listed more than once (replicas
// sharing its SMs).
void run_simulation(Config* cfg, GPUInfo* gpu, bool fp64_field) {
    const auto t_start = std::chrono::steady_clock::now();
    const int threadid = omp_get_thread_num ? omp_get_thread_num() : 0;
    if (threadid > 0) return;
    const int ndev = active_devices(cfg);
    if (ndev == 0) return;
    std::vector<int> ids(ndev);
    for (int d = 0; d < ndev; d++) {
        ids[d] = cfg->deviceid[d] - 1;
        if (ids[d] < 0) MCXG_RAISE(-1, "GPU ID must be non-zero");
    }
    const int gpuid = ids[0];
    if (cfg->debuglevel & kDebugRNG) {
        rng_debug_output(cfg, gpuid);
        return;
    }
    check_config(cfg);
    const std::vector<double> weights = device_weights(cfg, gpu, ndev);

    std::memset(&t_stats, 0, sizeof(t_stats));
    std::vector<std::unique_ptr<Session>> SS(ndev);
    for (auto& p : SS) p = std::make_unique<Session>();
    on_devices(ndev, [&](int d) { SS[d]->create(cfg, ids[d], fp64_field); });
    // every device holds the same gate group: the smallest any of them fits
    int maxgate = SS[0]->kp.maxgate;
    for (auto& p : SS) maxgate = std::min(maxgate, p->kp.maxgate);
    on_devices(ndev, [&](int d) {
        if (SS[d]->kp.maxgate != maxgate) {
            SS[d] = std::make_unique<Session>();
            SS[d]->create(cfg, ids[d], fp64_field, maxgate);
        }
    });
    Session& S = *SS[0];
    {
        // large runs tune the deposit tile with short pilot launches (cached per configuration)
        int tile_override;
        {
            std::lock_guard<std::mutex> g(g_override_mu);
            tile_override = g_override.tile;
        }
        const char* e = std::getenv("MCXG_TUNE");
        const bool tune = !(e && std::strcmp(e, "0") == 0);
        if (tune && tile_override < 0 && cfg->nphoton * (uint64_t)std::abs(cfg->respin) >= 20000000ull)
            on_devices(ndev, [&](int d) { SS[d]->autotune(cfg->nphoton); });
    }
    begin_outputs(cfg, S);
    const int reps = std::abs(cfg->respin);
    const uint64_t nper = (cfg->respin > 0) ? (uint64_t)cfg->nphoton : (uint64_t)cfg->nphoton / (uint64_t)reps;
    const uint64_t seed = (uint64_t)(uint32_t)cfg->seed;
    std::vector<uint64_t> offset, count;
    split_photons(weights, nper, offset, count);
    if (cfg->flog && cfg->printnum >= 0)
        for (int d = 0; d < ndev; d++)
            fprintf(cfg->flog, "GPU=%d (%s) np=%.0f grid=%d block=%d chunk=%d maxgate=%d repetition=%d\n", ids[d] + 1,
                    gpu ? gpu[ids[d]].name : "", (double)count[d] * (cfg->respin > 0 ? 1 : reps), SS[d]->grid,
                    SS[d]->block, SS[d]->kp.chunk, maxgate, reps);

    std::vector<float> host_field;
    mcxg_stats total{};
    std::vector<Session*> all;
    for (auto& p : SS) all.push_back(p.get());
    std::mutex mu;
    uint64_t run_index = 0;
    for (int gate0 = 0; gate0 < S.totalgates; gate0 += maxgate) {
        const float twin0 = cfg->tstart + cfg->tstep * gate0;
        on_devices(ndev, [&](int d) {
            Session& D = *SS[d];
            CK(cudaSetDevice(D.device));
            D.set_window(twin0, twin0 + cfg->tstep * maxgate);
            D.reset();
            // MCX seeds the generator of device thread d with seed + d (src/mcx_core.cu:3248)
            const uint64_t seed_d = (D.kp.seed_mode == 1) ? (uint64_t)(uint32_t)(cfg->seed + d) : seed;
            for (int it = 0; it < reps; it++) {
                if (D.savedet) CK(cudaMemsetAsync(D.detcount.p, 0, sizeof(unsigned), D.stream));
                if (D.kp.traj) CK(cudaMemsetAsync(D.trajcount.p, 0, sizeof(unsigned), D.stream));
                if (count[d]) D.run((run_index + it) * nper + offset[d], count[d], seed_d);
                append_detected(cfg, D, ndev > 1 ? &mu : nullptr);
                append_trajectory(cfg, D, ndev > 1 ? &mu : nullptr);
            }
        });
        run_index += reps;
        finish_window(cfg, all, host_field, total);
    }
    double kernel_ms = 0.0;
    int threads = 0;
    for (auto& p : SS) {
        kernel_ms = std::max(kernel_ms, p->kernel_ms);
        threads += p->grid * p->block;
    }
    total.kernel_ms = kernel_ms;
    total.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    t_stats = total;
    end_outputs(cfg, S, kernel_ms, reps, threads);
}

// Many independent simulations on one device (the batched workload): every Config gets its
// own session -- volume, media, source and field on the device -- and all transport launches
// go into one CUDA graph over `nstreams` streams, largest photon budget first.  A launch is a
// persistent grid drawing on its own photon counter, sized by its stream's share of the photons;
// as the CTAs of one launch run out of photons, the block scheduler fills the freed SMs with CTAs
// of the launches on the other streams, so the tail of one simulation overlaps the others.  Each
// Config's outputs are those of mcx_run_simulation; `runtime` is the batch's graph time.
constexpr int kMinBatchCTAs = 16;

// Oversubscription of the batched grids (CTAs requested over a full grid, summed over the streams
// of a wave), MCXG_BATCH_OVERSUB (1-16) when set.  Otherwise 2, or 1 for a wave of fewer than 20
// photons per thread of a full grid: there every CTA's life is a few photons long, and CTAs queued
// behind the first wave would mostly start only to find their simulation's photons taken
// (measured on 16 128^3 volumes: 64 against 70 ms at 11 photons per thread, 136 against 156 ms
// the other way at 31).
double batch_oversubscription(double photons_per_thread) {
    const char* e = std::getenv("MCXG_BATCH_OVERSUB");
    if (e) {
        const double v = std::atof(e);
        if (v >= 1.0 && v <= 16.0) return v;
    }
    return photons_per_thread < 20.0 ? 1.0 : 2.0;
}

void run_batch(Config** cfgs, int count, int nstreams, mcxg_stats* stats, double* graph_ms, float* const* dev_fields = nullptr) {
    if (count <= 0 || !cfgs) MCXG_RAISE(-4, "an empty batch");
    nstreams = std::max(1, std::min(nstreams, 32));
    const int gpuid = cfgs[0]->deviceid[0] - 1;
    if (gpuid < 0) MCXG_RAISE(-1, "GPU ID must be non-zero");
    // Each simulation runs |respin| repetitions in each of its gate groups, as mcx_run_simulation
    // does; the batch runs them in waves, wave w holding every simulation's w-th (group,
    // repetition), each wave one CUDA graph over all its simulations.
    std::vector<std::unique_ptr<Session>> S(count);
    std::vector<int> reps(count), groups(count);
    std::vector<uint64_t> nper(count);
    std::vector<mcxg_stats> totals(count);
    int waves = 0;
    for (int i = 0; i < count; i++) {
        Config* cfg = cfgs[i];
        check_config(cfg);
        S[i] = std::make_unique<Session>();
        S[i]->create(cfg, gpuid, false);
        reps[i] = std::abs(cfg->respin);
        groups[i] = (S[i]->totalgates + S[i]->kp.maxgate - 1) / S[i]->kp.maxgate;
        nper[i] = (cfg->respin > 0) ? (uint64_t)cfg->nphoton : (uint64_t)cfg->nphoton / (uint64_t)reps[i];
        waves = std::max(waves, reps[i] * groups[i]);
        const bool on_device = dev_fields && dev_fields[i];
        if (on_device && (reps[i] * groups[i] != 1 || !cfg->issave2pt))
            MCXG_RAISE(-4, "a field on the device needs a fluence output in one repetition of one gate group");
        begin_outputs(cfg, *S[i], !on_device);
        std::memset(&totals[i], 0, sizeof(mcxg_stats));
    }
    for (auto& s : S) CK(cudaStreamSynchronize(s->stream));

    std::vector<int> full_grid(count);
    for (int i = 0; i < count; i++) full_grid[i] = S[i]->grid;
    std::vector<int> order(count);
    for (int i = 0; i < count; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cfgs[a]->nphoton > cfgs[b]->nphoton; });

    std::vector<cudaStream_t> st(nstreams, nullptr);
    std::vector<cudaEvent_t> joins(nstreams, nullptr);
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto drop_graph = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    };
    auto cleanup = [&]() {
        drop_graph();
        for (auto e : joins) if (e) cudaEventDestroy(e);
        for (auto x : st) if (x) cudaStreamDestroy(x);
        if (fork) cudaEventDestroy(fork);
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        if (origin) cudaStreamDestroy(origin);
    };
    double total_ms = 0.0;
    std::vector<float> host_field;
    try {
        CK(cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        CK(cudaEventCreate(&t0));
        CK(cudaEventCreate(&t1));
        for (int k = 0; k < nstreams; k++) {
            CK(cudaStreamCreateWithFlags(&st[k], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&joins[k], cudaEventDisableTiming));
        }
        for (int w = 0; w < waves; w++) {
            // host-side set-up of this wave: gate window and MCX seed words per simulation
            for (int i = 0; i < count; i++) {
                if (w >= reps[i] * groups[i]) continue;
                const Config* cfg = cfgs[i];
                const int g = w / reps[i];
                if (w % reps[i] == 0) {
                    const float twin0 = cfg->tstart + cfg->tstep * g * S[i]->kp.maxgate;
                    S[i]->set_window(twin0, twin0 + cfg->tstep * S[i]->kp.maxgate);
                }
                if (S[i]->kp.seed_mode == 1) S[i]->mcx_seed_words((uint64_t)(uint32_t)cfg->seed);
            }
            for (auto& s : S) CK(cudaStreamSynchronize(s->stream));
            // CTAs of each launch: its stream's share of the wave's photons, times the
            // oversubscription (one or two), of a full grid.  A launch whose photons are fewer
            // than its threads holds every CTA until the longest photon of that CTA ends, so full
            // grids would run such simulations one after the other, each at its latency; shared
            // out, the launches of all streams are resident together and the oversubscribed CTAs
            // take the SMs that early finishers free.
            std::vector<int> stream_of(count, -1);
            std::vector<double> load(nstreams, 0.0);
            int slot = 0;
            for (int j = 0; j < count; j++) {
                const int i = order[j];
                if (w >= reps[i] * groups[i]) continue;
                stream_of[i] = slot++ % nstreams;
                load[stream_of[i]] += (double)nper[i];
            }
            double wave_load = 0.0;
            for (double l : load) wave_load += l;
            double threads = 0.0;           // of one full grid (the largest any simulation of the wave has)
            for (int i = 0; i < count; i++)
                if (stream_of[i] >= 0) threads = std::max(threads, (double)full_grid[i] * S[i]->block);
            const double over = batch_oversubscription(wave_load / std::max(1.0, threads));
            for (int i = 0; i < count; i++) {
                if (stream_of[i] < 0) continue;
                const double share = wave_load > 0.0 ? over * load[stream_of[i]] / wave_load : 1.0;
                const int full = full_grid[i];
                S[i]->grid = std::max(std::min(full, kMinBatchCTAs), std::min(full, (int)std::ceil(full * share)));
            }
            CK(cudaStreamBeginCapture(origin, cudaStreamCaptureModeRelaxed));
            CK(cudaEventRecord(fork, origin));
            for (int k = 0; k < nstreams; k++) CK(cudaStreamWaitEvent(st[k], fork, 0));
            for (int j = 0; j < count; j++) {
                const int i = order[j];
                if (stream_of[i] < 0) continue;
                const Config* cfg = cfgs[i];
                S[i]->enqueue(st[stream_of[i]], (uint64_t)w * nper[i], nper[i], (uint64_t)(uint32_t)cfg->seed,
                              w % reps[i] == 0);
            }
            for (int k = 0; k < nstreams; k++) {
                CK(cudaEventRecord(joins[k], st[k]));
                CK(cudaStreamWaitEvent(origin, joins[k], 0));
            }
            CK(cudaStreamEndCapture(origin, &graph));
            CK(cudaGraphInstantiate(&exec, graph, 0));
            CK(cudaEventRecord(t0, origin));
            CK(cudaGraphLaunch(exec, origin));
            CK(cudaEventRecord(t1, origin));
            CK(cudaEventSynchronize(t1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, t0, t1));
            total_ms += ms;
            drop_graph();
            for (int i = 0; i < count; i++) {
                if (w >= reps[i] * groups[i]) continue;
                append_detected(cfgs[i], *S[i]);
                append_trajectory(cfgs[i], *S[i]);
                if (w % reps[i] == reps[i] - 1)
                    finish_window(cfgs[i], {S[i].get()}, host_field, totals[i], dev_fields ? dev_fields[i] : nullptr);
            }
        }
        if (dev_fields)
            for (auto& s : S) CK(cudaStreamSynchronize(s->stream));     // the fields are complete on return
        if (graph_ms) *graph_ms = total_ms;
        for (int i = 0; i < count; i++) {
            totals[i].kernel_ms = total_ms;
            if (stats) stats[i] = totals[i];
            end_outputs(cfgs[i], *S[i], total_ms, reps[i]);
        }
    } catch (...) {
        cudaStreamEndCapture(origin, &graph);      // leaves capture mode if an error came mid-capture
        cleanup();
        throw;
    }
    cleanup();
}

}  // namespace

extern "C" int mcxg_run_batch(Config** cfgs, int count, int nstreams, mcxg_stats* stats, double* graph_ms) {
    mcxg_clear_error();
    try {
        run_batch(cfgs, count, nstreams, stats, graph_ms);
        return 0;
    } catch (const Error& e) {
        report(e);
        return e.id ? e.id : -1;
    }
}

extern "C" int mcxg_run_batch_device(Config** cfgs, int count, int nstreams, float* const* dev_fields, mcxg_stats* stats,
                                     double* graph_ms) {
    mcxg_clear_error();
    try {
        if (!dev_fields) MCXG_RAISE(-4, "no device fields given");
        run_batch(cfgs, count, nstreams, stats, graph_ms, dev_fields);
        return 0;
    } catch (const Error& e) {
        report(e);
        return e.id ? e.id : -1;
    }
}

extern "C" void mcx_run_simulation(Config* cfg, GPUInfo* gpu) {
    mcxg_clear_error();
    try {
        run_simulation(cfg, gpu, field_fp64());
    } catch (const Error& e) {
        report(e);
    }
}

// The photon split of mcx_run_simulation over the devices listed in cfg->deviceid.
extern "C" int mcxg_photon_shares(Config* cfg, const GPUInfo* gpu, uint64_t nphoton, uint64_t* offsets, uint64_t* counts) {
    mcxg_clear_error();
    try {
        const int ndev = active_devices(cfg);
        if (ndev == 0) return 0;
        std::vector<uint64_t> off, cnt;
        split_photons(device_weights(cfg, gpu, ndev), nphoton, off, cnt);
        for (int d = 0; d < ndev; d++) {
            offsets[d] = off[d];
            counts[d] = cnt[d];
        }
        return ndev;
    } catch (const Error& e) {
        mcxg_set_error(e.id ? e.id : -1, e.msg.c_str());
        return e.id ? e.id : -1;
    }
}

// Same run with the field accumulated in FP64 on the device: the reference-accuracy twin used
// to state the FP32 accumulation error of the production path.
extern "C" void mcxg_run_simulation_fp64(Config* cfg, GPUInfo* gpu) {
    mcxg_clear_error();
    try {
        run_simulation(cfg, gpu, true);
    } catch (const Error& e) {
        report(e);
    }
}

// ---------------------------------------------------------------------------------------------
// RNG test kernels
// ---------------------------------------------------------------------------------------------
extern "C" int mcxg_rng_test(const uint32_t seeds[4], float* out, int n) {
    mcxg_clear_error();
    try {
        uint32_t* ds = nullptr;
        float* dout = nullptr;
        CK(cudaMalloc(&ds, 16));
        CK(cudaMalloc(&dout, sizeof(float) * (size_t)std::max(n, 1)));
        CK(cudaMemcpy(ds, seeds, 16, cudaMemcpyHostToDevice));
        CK(launch_rng_test(ds, dout, n, 0));
        CK(cudaMemcpy(out, dout, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost));
        cudaFree(ds);
        cudaFree(dout);
        return 0;
    } catch (const Error& e) {
        report(e);
        return t_err_id;
    }
}

extern "C" int mcxg_photon_stream(uint64_t seed, uint64_t pid, float* out, int n) {
    mcxg_clear_error();
    try {
        float* dout = nullptr;
        CK(cudaMalloc(&dout, sizeof(float) * (size_t)std::max(n, 1)));
        CK(launch_photon_stream(seed, pid, dout, n, 0));
        CK(cudaMemcpy(out, dout, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost));
        cudaFree(dout);
        return 0;
    } catch (const Error& e) {
        report(e);
        return t_err_id;
    }
}

// Measured FP32 reduction throughput into L2 over `nfloats` distinct addresses (the
// deposit-bound denominator of the transport roofline), in reductions per second.
extern "C" int mcxg_probe_atomic_rate(uint64_t nfloats, double* per_second) {
    mcxg_clear_error();
    try {
        int dev = 0, sms = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        float* buf = nullptr;
        CK(cudaMalloc(&buf, nfloats * sizeof(float)));
        CK(cudaMemset(buf, 0, nfloats * sizeof(float)));
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        const int block = 256, grid = sms * 8, iters = 256;
        CK(launch_atomic_probe(buf, (unsigned)nfloats, iters, grid, block, 0));   // warm-up
        CK(cudaEventRecord(a, 0));
        CK(launch_atomic_probe(buf, (unsigned)nfloats, iters, grid, block, 0));
        CK(cudaEventRecord(b, 0));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        cudaFree(buf);
        *per_second = (double)grid * block * iters / (ms * 1e-3);
        return 0;
    } catch (const Error& e) {
        report(e);
        return t_err_id;
    }
}

// ---------------------------------------------------------------------------------------------
// Sessions
// ---------------------------------------------------------------------------------------------
struct mcxg_session {
    Session s;
};

extern "C" mcxg_session* mcxg_session_create(const Config* cfg, int device) {
    mcxg_clear_error();
    mcxg_session* h = new mcxg_session();
    try {
        h->s.create(cfg, device, false);
        h->s.set_window(cfg->tstart, cfg->tstart + cfg->tstep * h->s.kp.maxgate);
        return h;
    } catch (const Error& e) {
        delete h;
        report(e);
        return nullptr;
    }
}

extern "C" int mcxg_session_reset(mcxg_session* h) {
    try {
        h->s.reset();
        return 0;
    } catch (const Error& e) {
        report(e);
        return t_err_id;
    }
}

extern "C" int mcxg_session_run(mcxg_session* h, uint64_t photon_offset, uint64_t nphoton, uint64_t seed, float* kernel_ms) {
    try {
        const float ms = h->s.run(photon_offset, nphoton, seed);
        if (kernel_ms) *kernel_ms = ms;
        return 0;
    } catch (const Error& e) {
        report(e);
        return t_err_id;
    }
}

extern "C" int64_t mcxg_session_read(mcxg_session* h, float* field, float* detp, uint64_t max_records, mcxg_stats* stats) {
    try {
        Session& s = h->s;
        if (field) s.read_field(field, 1.f, 0);
        const unsigned det = s.detected();
        if (detp && s.detp.p && det) {
            const uint64_t n = std::min<uint64_t>(std::min<uint64_t>(det, s.kp.maxdet), max_records);
            CK(cudaMemcpyAsync(detp, s.detp.p, n * s.kp.reclen * sizeof(float), cudaMemcpyDeviceToHost, s.stream));
            CK(cudaStreamSynchronize(s.stream));
        }
        if (stats) s.read_stats(stats);
        return (int64_t)det;
    } catch (const Error& e) {
        report(e);
        return (int64_t)t_err_id;
    }
}

extern "C" void mcxg_session_destroy(mcxg_session* h) { delete h; }

extern "C" int mcxg_session_autotune(mcxg_session* h, uint64_t nphoton) {
    try {
        h->s.autotune(nphoton);
        return 0;
    } catch (const Error& e) {
        report(e);
        return t_err_id;
    }
}
