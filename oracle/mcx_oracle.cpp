// mcx_oracle.cpp -- CPU restatement of MCX's voxel photon-transport loop.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle and the CPU baseline of the
// GB300 engine; the engine never calls it.  Only tests/, the smoke check in
// __graft_entry__.py and the cpu_baseline leg of bench.py load it, and only as a checker.
//
// What it restates (MCX v2025.10, file:line within the reference project):
//   xorshift128+ generator ............ src/mcx_rand_xorshift128p.cu:56-82, 109-138
//   RNG test kernel (-D R) ............ src/mcx_core.cu:1731-1742
//   mcx_nextafterf .................... src/mcx_core.cu:470-478
//   hitgrid ........................... src/mcx_core.cu:493-507
//   transmit .......................... src/mcx_core.cu:523-537
//   reflectcoeff ...................... src/mcx_core.cu:552-570
//   skipvoid (label media) ............ src/mcx_core.cu:866-956
//   rotatevector ...................... src/mcx_core.cu:1011-1031
//   launchnewphoton (pencil branch) ... src/mcx_core.cu:1089-1243, 1646-1717
//   savedetphoton / finddetector ...... src/mcx_core.cu:258-270, 365-417
//   mcx_main_loop<1,r,1,0,0> .......... src/mcx_core.cu:1767-2528
//   split voxels (MEDIA_2LABEL_SPLIT) . src/mcx_core.cu:688-830 (updateproperty, ray_plane_intersect,
//                                        reflectray), 2112-2133, 2295-2310, 2386-2404, 2474-2507
//   extra sources ..................... src/mcx_core.cu:1217-1227 (source draw), 2225-2227 (blocks),
//                                        383 (source in the detector id); src/mcx_utils.c:1688-1692
// The control flow follows the reference step for step, in plain FP32 with libm's
// logf/expf/sincosf/acosf/sinf standing in for the CUDA fast-math intrinsics the reference
// is compiled with.  Differences that are deliberate:
//   * RNG seeding: every photon gets its own xorshift128+ state derived from (seed, photon
//     index) by the splitmix64 mixer, exactly as the GB300 engine seeds it.  The reference
//     seeds one state per GPU thread from glibc rand(); streams therefore differ, statistics
//     do not.  The generator itself is pinned bit-for-bit by tests/golden (the -D R vector).
//   * Tallies are FP64 (field, energies) so the oracle carries no FP32 accumulation error;
//     it also counts steps, scatters, deposits and per-voxel deposit hits, the algorithmic
//     quantities the roofline is built from.
// Parity is pinned against the reference's own golden numbers (absorbed fraction of cube60 /
// cube60b, detected-photon count of cube60b, the RNG vector) and against the semi-infinite
// CW diffusion solution; see tests/test_oracle_golden.py.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <chrono>
#include <cstdlib>
#include <vector>
#include <atomic>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mcx_oracle.h"

namespace {

constexpr float kEPS = FLT_EPSILON;
constexpr uint32_t kDET_MASK = 0x80000000u;
constexpr uint32_t kMED_MASK = 0x7FFFFFFFu;
constexpr uint32_t kOUT_MIN = 0xFFFFFFFFu;   // left the volume through x/y/z = 0 side
constexpr uint32_t kOUT_MAX = 0x7FFFFFFFu;   // left through the far side
constexpr float kTWO_PI = 6.28318530717959f;
constexpr float kR_C0 = 3.335640951981520e-12f;  // s/mm
enum { BC_UNKNOWN = 0, BC_REFLECT = 1, BC_ABSORB = 2, BC_MIRROR = 3, BC_CYCLIC = 4 };

// ---------------------------------------------------------------- xorshift128+ ----------
struct Rng {
    uint64_t s[2];
    // src/mcx_rand_xorshift128p.cu:56-72: one step; the float is built from the low 32 bits
    float next() {
        uint64_t s1 = s[0];
        const uint64_t s0 = s[1];
        s[0] = s0;
        s1 ^= s1 << 23;
        s[1] = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
        uint32_t lo = (uint32_t)(s[1] + s0);
        uint32_t bits = 0x3F800000u | (lo >> 9);
        float f;
        std::memcpy(&f, &bits, 4);
        return f - 1.0f;
    }
};

inline uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-photon seeding shared with the GB300 engine (mcx_gb300/csrc/rng.cuh).
inline void seed_photon(Rng& r, uint64_t seed, uint64_t photon) {
    uint64_t x = seed * 0xD1B54A32D192ED03ull + photon;
    r.s[0] = splitmix64(x);
    r.s[1] = splitmix64(x);
    if ((r.s[0] | r.s[1]) == 0) r.s[1] = 1;
}

struct Prop { float mua, mus, g, n; };

struct Ctx {
    const OracleProblem* P;
    uint32_t nx, ny, nz, dimxy, dimxyz;
    float maxx, maxy, maxz;
    float oneoverc0, minaccumtime, Rtstep, twin0, twin1;
    uint32_t maxgate, medianum, detnum;
    uint32_t partialdata, reclen;
    int isreflect;                 // template flag of the reference (isreflect or any r/m face)
    const Prop* prop;

    // Properties of a voxel's medium value m: the table row for labels; for the per-voxel formats
    // decoded from the word, the fields a format does not store taken from row 1 (MCX's kernel
    // starts from row 1 and never overwrites them), n from row 1 (src/mcx_core.cu:614-695).  A
    // void or outside voxel (m = 0) takes row 0 in every format, unlike MCX's decode of a zero
    // MEDIA_ASGN_BYTE word (the engine's rule, restated here).
    Prop prop_of(uint32_t m, uint32_t idx) const {
        const int f = P->mediaformat;
        if (f <= 4 || m == 0) return prop[m];
        if (f == 98) return prop[m & 0xFF];        // a mixed voxel resolved to one label (pick)
        if (f == 96) {      // src/mcx_core.cu:628-647: [mus][mua] halves, [n][g] in the second word
            const uint32_t m2 = P->vol[(size_t)dimxy * nz + idx];
            return {std::fabs(half_to_float(m & 0xFFFF)), std::fabs(half_to_float(m >> 16)),
                    std::fabs(half_to_float(m2 & 0xFFFF)), std::fabs(half_to_float(m2 >> 16))};
        }
        if (f == 99) {      // src/mcx_core.cu:597-613: the label's row with one field replaced
            Prop r = prop[m & 0x3FFF];
            const float v = std::fabs(half_to_float(m >> 16));
            const uint32_t fld = (m >> 14) & 3;
            if (fld == 0) r.mua = v;
            else if (fld == 1) r.mus = v;
            else if (fld == 2) r.g = v;
            else r.n = v;
            return r;
        }
        const Prop r1 = prop[1];
        const float n = r1.n;
        if (f == 101) {
            float mua;
            std::memcpy(&mua, &m, 4);
            return {std::fabs(mua), r1.mus, r1.g, n};
        }
        if (f == 100 || f == 102) return {std::fabs(half_to_float(m & 0xFFFF)), std::fabs(half_to_float(m >> 16)), r1.g, n};
        const Prop r2 = prop[2];
        if (f == 103)
            return {(m & 0xFF) * (1.f / 255.f) * (r2.mua - r1.mua) + r1.mua, ((m >> 8) & 0xFF) * (1.f / 255.f) * (r2.mus - r1.mus) + r1.mus,
                    ((m >> 16) & 0xFF) * (1.f / 255.f) * (r2.g - r1.g) + r1.g, (m >> 24) * (1.f / 127.f) * (r2.n - r1.n) + r1.n};
        return {(m & 0xFFFF) * (1.f / 65535.f) * (r2.mua - r1.mua) + r1.mua, (m >> 16) * (1.f / 65535.f) * (r2.mus - r1.mus) + r1.mus,
                r1.g, n};
    }

    // MEDIA_2LABEL_SPLIT (src/mcx_core.cu:688-730): the voxel's first word holds [lower][upper]
    // [point x][point y], its second (after all first words) [point z][normal x][normal y]
    // [normal z], bytes over 0..1 of the voxel and -1..1 of the normal (mcx_preprocess's layout,
    // src/mcx_utils.c:1708-1731).  Sets the photon's split-voxel state for its voxel and position
    // and returns the properties of the tissue it is in; outside the volume row 0, state kept.
    template <class PH>
    Prop svmc_prop(PH& ph) const {
        if (ph.idx1d == 0xFFFFFFFFu || ph.idx1d == 0x7FFFFFFFu) return prop[0];
        const uint32_t w1 = P->vol[ph.idx1d] & 0x7FFFFFFFu, w0 = P->vol[(size_t)dimxyz + ph.idx1d];
        ph.sv_lo = (int)(w1 >> 24);
        ph.sv_up = (int)((w1 >> 16) & 0xFFu);
        if (ph.sv_up) {
            ph.rp[0] = ((w1 >> 8) & 0xFFu) * (1.f / 255.f) + ph.fd[0];
            ph.rp[1] = (w1 & 0xFFu) * (1.f / 255.f) + ph.fd[1];
            ph.rp[2] = (w0 >> 24) * (1.f / 255.f) + ph.fd[2];
            float n[3] = {((w0 >> 16) & 0xFFu) * (2.f / 255.f) - 1, ((w0 >> 8) & 0xFFu) * (2.f / 255.f) - 1,
                          (w0 & 0xFFu) * (2.f / 255.f) - 1};
            const float inv = 1.f / std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int i = 0; i < 3; i++) ph.nv[i] = n[i] * inv;
            const float side = (ph.rp[0] - ph.p[0]) * ph.nv[0] + (ph.rp[1] - ph.p[1]) * ph.nv[1] +
                               (ph.rp[2] - ph.p[2]) * ph.nv[2];
            ph.sv_split = true;
            if (side < 0.f) {            // the upper tissue; the normal always points to the other side
                ph.sv_isup = true;
                for (int i = 0; i < 3; i++) ph.nv[i] = -ph.nv[i];
                return prop[ph.sv_up];
            }
            ph.sv_isup = false;
            return prop[ph.sv_lo];
        }
        ph.sv_split = false;
        ph.sv_isup = false;
        return prop[ph.sv_lo];
    }

    // MEDIA_2LABEL_MIX (src/mcx_core.cu:649-666): a word [15-bit fraction][label 1][label 0] is
    // label 1 with probability fraction / 32767, else label 0, drawn when the photon enters the
    // voxel; the detector bit is kept.  Other formats pass through.
    template <class R>
    uint32_t pick(uint32_t w, R& rng) const {
        if (P->mediaformat != 98) return w;
        const uint32_t frac = (w >> 16) & 0x7FFF;
        uint32_t c = w & 0xFF;
        if (frac > 0 && rng.next() * 32767.f < (float)frac) c = (w >> 8) & 0xFF;
        return (w & kDET_MASK) | c;
    }

    // IEEE 754 binary16 bits to float (normals, subnormals, zero; the formats store no inf/NaN)
    static float half_to_float(uint32_t h) {
        const uint32_t sign = (h >> 15) & 1u, e = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
        float v;
        if (e == 0) v = std::ldexp((float)man, -24);
        else v = std::ldexp((float)(man | 0x400u), (int)e - 25);
        return sign ? -v : v;
    }
};

// src/mcx_core.cu:470-478
inline float nextafter_mcx(float a, int dir, float maxvoidstep) {
    float f = a + maxvoidstep;
    uint32_t i;
    std::memcpy(&i, &f, 4);
    i += (uint32_t)dir ^ (i & 0x80000000u);
    std::memcpy(&f, &i, 4);
    return f - maxvoidstep;
}

// src/mcx_core.cu:493-507
inline float hitgrid(const float p[3], const float v[3], const float rv[3], short fd[4]) {
    float h0 = std::fabs((fd[0] + (v[0] > 0.f) - p[0]) * rv[0]);
    float h1 = std::fabs((fd[1] + (v[1] > 0.f) - p[1]) * rv[1]);
    float h2 = std::fabs((fd[2] + (v[2] > 0.f) - p[2]) * rv[2]);
    float d = std::fmin(std::fmin(h0, h1), h2);
    fd[3] = (d == h0 ? 0 : (d == h1 ? 1 : 2));
    return d;
}

// src/mcx_core.cu:523-537
inline void transmit(float v[3], float n1, float n2, int axis) {
    float t = n1 / n2;
    v[0] *= t; v[1] *= t; v[2] *= t;
    int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
    float s = v[a1] * v[a1] + v[a2] * v[a2];
    v[axis] = (s < 1.f) ? std::sqrt(1.f - s) * (float)((v[axis] > 0.f) - (v[axis] < 0.f)) : 0.f;
    float r = 1.f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= r; v[1] *= r; v[2] *= r;
}

// src/mcx_core.cu:552-570
inline float reflectcoeff(const float v[3], float n1, float n2, int axis) {
    float Icos = std::fabs(v[axis]);
    float a = n1 * n1, b = n2 * n2;
    float c = 1.f - a / b * (1.f - Icos * Icos);
    if (c > 0.f) {
        float Re = a * Icos * Icos + b * c;
        c = std::sqrt(c);
        float Im = 2.f * n1 * n2 * Icos * c;
        float R = (Re - Im) / (Re + Im);
        Re = b * Icos * Icos + a * c * c;
        return (R + (Re - Im) / (Re + Im)) * 0.5f;
    }
    return 1.f;
}

// src/mcx_core.cu:1011-1031
inline void rotatevector(float v[3], float st, float ct, float sp, float cp) {
    if (v[2] > -1.f + kEPS && v[2] < 1.f - kEPS) {
        float t0 = 1.f - v[2] * v[2];
        float t1 = st / std::sqrt(t0);
        float nx = t1 * (v[0] * v[2] * cp - v[1] * sp) + v[0] * ct;
        float ny = t1 * (v[1] * v[2] * cp + v[0] * sp) + v[1] * ct;
        float nz = -t1 * t0 * cp + v[2] * ct;
        v[0] = nx; v[1] = ny; v[2] = nz;
    } else {
        float nz = (v[2] > 0.f) ? ct : -ct;
        v[0] = st * cp; v[1] = st * sp; v[2] = nz;
    }
    float r = 1.f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= r; v[1] *= r; v[2] *= r;
}

inline bool inside(const Ctx& C, const short fd[4]) {
    return (unsigned short)fd[0] < C.maxx && (unsigned short)fd[1] < C.maxy && (unsigned short)fd[2] < C.maxz;
}

inline uint32_t vidx(const Ctx& C, const short fd[4]) {
    return (uint32_t)(fd[2] * (int)C.dimxy + fd[1] * (int)C.nx + fd[0]);
}

struct Tally {
    double e_launch = 0, e_escape = 0, e_detect = 0, e_absdep = 0, e_absother = 0;
    uint64_t steps = 0, scatters = 0, deposits = 0, launches = 0, detected = 0, photons = 0;
};

struct Photon {
    float p[3], w;
    float v[3], nscat;
    float pscat, t, pathlen;
    float w0, wlaunch;
    float rv[3];
    short fd[4];
    uint32_t idx1d, mediaid;
    int isdet;
    Prop prop;
    float ppath[3 * 128];          // nscat(M) | ppath(M) | mom(M), per medium label 1..M
    // split voxel of the current position (MEDIA_2LABEL_SPLIT, src/mcx_core.cu:688-730): the two
    // labels, the plane's point and its normal turned toward the other tissue, the side the photon
    // is on, and whether the next flight tests the plane
    int sv_lo, sv_up;
    bool sv_split, sv_isup, testint;
    float rp[3], nv[3];
    int src;                       // 1-based source of the photon (extra sources)
};

// src/mcx_core.cu:866-956 (label media, no SVMC).  Returns the entry voxel or -1.
int skipvoid(const Ctx& C, Photon& ph) {
    const OracleProblem* P = C.P;
    int count = 1;
    short fd[4] = {0, 0, 0, -1};
    fd[0] = (short)std::floor(ph.p[0]);
    fd[1] = (short)std::floor(ph.p[1]);
    fd[2] = (short)std::floor(ph.p[2]);
    while (true) {
        if (inside(C, fd)) {
            uint32_t id = vidx(C, fd);
            if (P->vol[id] & kMED_MASK) {
                ph.p[0] -= ph.v[0]; ph.p[1] -= ph.v[1]; ph.p[2] -= ph.v[2];
                fd[0] = (short)std::floor(ph.p[0]);
                fd[1] = (short)std::floor(ph.p[1]);
                fd[2] = (short)std::floor(ph.p[2]);
                ph.t -= C.minaccumtime;
                id = vidx(C, fd);
                count = 0;
                while (!inside(C, fd) || !(P->vol[id] & kMED_MASK)) {
                    float d = hitgrid(ph.p, ph.v, ph.rv, fd);
                    ph.t += C.minaccumtime * d;
                    ph.p[0] += d * ph.v[0]; ph.p[1] += d * ph.v[1]; ph.p[2] += d * ph.v[2];
                    if (fd[3] == 0) fd[0] += (ph.v[0] > 0.f ? 1 : -1);
                    if (fd[3] == 1) fd[1] += (ph.v[1] > 0.f ? 1 : -1);
                    if (fd[3] == 2) fd[2] += (ph.v[2] > 0.f ? 1 : -1);
                    id = vidx(C, fd);
                    if (count++ > 3) break;
                }
                ph.t = P->voidtime ? ph.t : 0.f;
                const Prop np = C.prop_of(P->vol[id] & kMED_MASK, (uint32_t)id);
                if (P->isspecular && np.n != C.prop[0].n) {
                    ph.w *= 1.f - reflectcoeff(ph.v, C.prop[0].n, np.n, fd[3]);
                    if (ph.w > kEPS) transmit(ph.v, C.prop[0].n, np.n, fd[3]);
                }
                return (int)id;
            }
        }
        if ((ph.p[0] < 0.f && ph.v[0] <= 0.f) || (ph.p[0] >= C.maxx && ph.v[0] >= 0.f) ||
            (ph.p[1] < 0.f && ph.v[1] <= 0.f) || (ph.p[1] >= C.maxy && ph.v[1] >= 0.f) ||
            (ph.p[2] < 0.f && ph.v[2] <= 0.f) || (ph.p[2] >= C.maxz && ph.v[2] >= 0.f))
            return -1;
        ph.p[0] += ph.v[0]; ph.p[1] += ph.v[1]; ph.p[2] += ph.v[2];
        fd[0] = (short)std::floor(ph.p[0]);
        fd[1] = (short)std::floor(ph.p[1]);
        fd[2] = (short)std::floor(ph.p[2]);
        ph.t += C.minaccumtime;
        if (count++ > P->maxvoidstep) return -1;
    }
}

// src/mcx_core.cu:258-270
uint32_t finddetector(const Ctx& C, const float p[3]) {
    for (uint32_t i = 0; i < C.detnum; i++) {
        const float* d = C.P->detpos + 4 * i;
        if ((d[0] - p[0]) * (d[0] - p[0]) + (d[1] - p[1]) * (d[1] - p[1]) + (d[2] - p[2]) * (d[2] - p[2]) < d[3] * d[3])
            return (d[3] < 0.f) ? 0 : i + 1;
    }
    return 0;
}

// src/mcx_core.cu:365-417 (savedetflag fields D,S,P,M,X,V,W; no seeds, no Stokes)
void savedetphoton(const Ctx& C, OracleResult* R, std::atomic<uint64_t>& slot, const Photon& ph, uint32_t isdet, Tally& T) {
    int detid = (isdet == kOUT_MIN) ? -1 : (int)finddetector(C, ph.p);
    if (!detid) return;
    T.detected++;
    uint64_t base = slot.fetch_add(1);
    if (base >= C.P->maxdetphoton || !R->detp) return;
    float* rec = R->detp + base * C.reclen;
    uint32_t k = 0, flag = C.P->savedetflag;
    if (flag & 0x1) rec[k++] = (float)((C.P->nextra && C.P->srcid <= 0) ? (detid | (ph.src << 16)) : detid);
    for (uint32_t i = 0; i < C.partialdata; i++) rec[k++] = ph.ppath[i];
    if (flag & 0x10) { rec[k++] = ph.p[0]; rec[k++] = ph.p[1]; rec[k++] = ph.p[2]; }
    if (flag & 0x20) { rec[k++] = ph.v[0]; rec[k++] = ph.v[1]; rec[k++] = ph.v[2]; }
    if (flag & 0x40) rec[k++] = ph.wlaunch;
}

struct Runner {
    Ctx C;
    OracleResult* R;
    std::atomic<uint64_t>* detslot;
    const OracleProblem* srcs = nullptr;   // source k's problem at srcs[k - 1]: the primary, then the extras

    void deposit(uint32_t idx, int tshift, double val) {
        double* f = R->field + (size_t)idx + (size_t)tshift * C.dimxyz;
#pragma omp atomic
        *f += val;
        if (R->hits) {
            uint64_t* h = R->hits + (size_t)idx + (size_t)tshift * C.dimxyz;
#pragma omp atomic
            *h += 1;
        }
    }

    // Terminate the current photon (energy and detection bookkeeping, src/mcx_core.cu:1113-1182).
    void terminate(Photon& ph, uint32_t isdet, Tally& T) {
        const OracleProblem* P = C.P;
        bool det = false;
        if (P->savedet && (isdet & kDET_MASK) == kDET_MASK && ph.mediaid == 0) {
            uint64_t before = T.detected;
            savedetphoton(C, R, *detslot, ph, isdet, T);
            det = T.detected != before;
        }
        if (det) T.e_detect += ph.w; else T.e_escape += ph.w;
        // absorption since the last recorded deposit is not in the field
        T.e_absother += (double)ph.w0 - (double)ph.w;
    }

    // Launch a pencil-beam photon (src/mcx_core.cu:1236-1243, 1646-1717).  Returns false on failure.
    // Shape of a non-pencil source: position, weight and direction of one photon, drawn in the
    // reference's order (launchnewphoton, src/mcx_core.cu:1261-1640; no launch-angle table).
    // Sets the launch voxel for shapes that move the photon.  False when the weight is at or
    // below minenergy (the reference then draws again without counting an attempt).
    bool sample_source(Photon& ph, Rng& rng, const OracleProblem* P) {
        const float* a = P->srcparam1;
        const float* b = P->srcparam2;
        const float W = P->srcpos[3];
        const float kJBO = 0.9998f;            // JUST_BELOW_ONE, src/mcx_const.h:50
        float origin[3] = {P->srcpos[0], P->srcpos[1], P->srcpos[2]};
        bool canfocus = true, moved = true;
        auto U = [&]() { return rng.next(); };
        auto scatlen = [&]() { return -std::log(rng.next() + kEPS); };
        auto rotate_to = [&](float st, float ct, float sp, float cp) { rotatevector(ph.v, st, ct, sp, cp); };
        switch (P->srctype) {
        case 4: case 5: case 15: case 6: case 14: {          // planar, pattern, pattern3d, fourier, pencilarray
            const float rx = U(), ry = U();
            if (P->srctype == 15) {
                const float rz = U();
                ph.p[0] += rx * a[0]; ph.p[1] += ry * a[1]; ph.p[2] += rz * a[2];
                const int nx = (int)a[0], ny = (int)a[1];
                ph.w = W * P->srcpattern[(int)(rz * kJBO * a[2]) * ny * nx + (int)(ry * kJBO * a[1]) * nx + (int)(rx * kJBO * a[0])];
            } else {
                for (int i = 0; i < 3; i++) ph.p[i] += rx * a[i] + ry * b[i];
                if (P->srctype == 5) {
                    ph.w = W * P->srcpattern[(int)(ry * kJBO * b[3]) * (int)a[3] + (int)(rx * kJBO * a[3])];
                } else if (P->srctype == 6) {
                    ph.w = W * (std::cos((std::floor(a[3]) * rx + std::floor(b[3]) * ry + a[3] - std::floor(a[3])) * kTWO_PI) *
                                    (1.f - b[3] + std::floor(b[3])) + 1.f) * 0.5f;
                } else if (P->srctype == 14) {
                    const float i = std::floor(rx * a[3]) / (a[3] - 1.f), j = std::floor(ry * b[3]) / (b[3] - 1.f);
                    for (int k = 0; k < 3; k++) ph.p[k] = P->srcpos[k] + i * a[k] + j * b[k];
                }
            }
            for (int i = 0; i < 3; i++) origin[i] += (a[i] + b[i]) * 0.5f;
            break;
        }
        case 9: case 10: {                                     // fourierx, fourierx2d
            const float rx = U(), ry = U();
            const float s = a[3] / std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
            const float d[3] = {P->srcdir[0], P->srcdir[1], P->srcdir[2]};
            const float v2[3] = {s * (d[1] * a[2] - d[2] * a[1]), s * (d[2] * a[0] - d[0] * a[2]), s * (d[0] * a[1] - d[1] * a[0])};
            for (int i = 0; i < 3; i++) ph.p[i] += rx * a[i] + ry * v2[i];
            if (P->srctype == 10)
                ph.w = W * (std::sin((b[0] * rx + b[2]) * kTWO_PI) * std::sin((b[1] * ry + b[3]) * kTWO_PI) + 1.f) * 0.5f;
            else
                ph.w = W * (std::cos((b[0] * rx + b[1] * ry + b[2]) * kTWO_PI) * (1.f - b[3]) + 1.f) * 0.5f;
            for (int i = 0; i < 3; i++) origin[i] += (a[i] + v2[i]) * 0.5f;
            break;
        }
        case 8: case 17: case 3: {                             // disk, ring, gaussian
            const float phi = (P->srctype == 17 && (a[2] > 0.f || a[3] > 0.f))
                                  ? std::fabs(a[2] - a[3]) * U() + std::fmin(a[2], a[3]) : kTWO_PI * U();
            const float sp = std::sin(phi), cp = std::cos(phi);
            float r;
            if (P->srctype != 3) {
                r = std::sqrt(U() * std::fabs(a[0] * a[0] - a[1] * a[1]) + a[1] * a[1]);
            } else if (std::fabs(P->srcdir[3]) < 1e-5f || std::fabs(a[1]) < 1e-5f) {
                r = std::sqrt(0.5f * scatlen()) * a[0];
            } else {
                const float zr = a[0] * a[0] * 3.14159265358979f / a[1];
                r = std::sqrt(0.5f * scatlen() * (1.f + P->srcdir[3] * P->srcdir[3] / (zr * zr))) * a[0];
            }
            const float* v = ph.v;
            if (v[2] > -1.f + kEPS && v[2] < 1.f - kEPS) {
                const float t0 = 1.f - v[2] * v[2], t1 = r / std::sqrt(t0);
                ph.p[0] += t1 * (v[0] * v[2] * cp - v[1] * sp);
                ph.p[1] += t1 * (v[1] * v[2] * cp + v[0] * sp);
                ph.p[2] -= t1 * t0 * cp;
            } else {
                ph.p[0] += r * cp;
                ph.p[1] += r * sp;
            }
            break;
        }
        case 2: case 1: case 7: {                              // cone, isotropic, arcsine
            float ang = kTWO_PI * U();
            const float sp = std::sin(ang), cp = std::cos(ang);
            if (P->srctype == 2) {
                const float c = std::cos(a[0]);
                ang = (a[1] > 0.f) ? U() * a[0] : std::acos(U() * (1.f - c) + c);
            } else if (P->srctype == 1) {
                ang = std::acos(2.f * U() - 1.f);
            } else {
                ang = 3.14159265358979f * U();
            }
            rotate_to(std::sin(ang), std::cos(ang), sp, cp);
            canfocus = false;
            moved = false;
            break;
        }
        case 11: {                                             // zgaussian
            float ang = kTWO_PI * U();
            const float sp = std::sin(ang), cp = std::cos(ang);
            ang = std::sqrt(2.f * scatlen());
            ang *= (1.f - 2.f * U()) * a[0];
            rotate_to(std::sin(ang), std::cos(ang), sp, cp);
            canfocus = false;
            moved = false;
            break;
        }
        case 16: {                                             // hyperboloid gaussian
            const float phi = kTWO_PI * U();
            const float sp = std::sin(phi), cp = std::cos(phi);
            const float r = std::sqrt(0.5f * scatlen()) * a[0];
            const float q = -a[1] / a[2], k = 1.f / std::sqrt(r * r + a[2] * a[2]);
            float d[3] = {r * (cp - q * sp), r * (sp + q * cp), 0.f};           // displacement
            const float u[3] = {-r * sp * k, r * cp * k, a[2] * k};            // direction, beam frame
            const float* v = ph.v;
            if (v[2] > -1.f + kEPS && v[2] < 1.f - kEPS) {
                const float st = std::sqrt(1.f - v[2] * v[2]);
                const float c = v[0] / st, s_ = v[1] / st, vz = v[2];
                const float dd[3] = {d[0] * c * vz - d[1] * s_, d[0] * s_ * vz + d[1] * c, -d[0] * st};
                ph.v[0] = u[0] * c * vz - u[1] * s_ + u[2] * c * st;
                ph.v[1] = u[0] * s_ * vz + u[1] * c + u[2] * s_ * st;
                ph.v[2] = -u[0] * st + u[2] * vz;
                d[0] = dd[0]; d[1] = dd[1]; d[2] = dd[2];
            } else {
                ph.v[0] = u[0]; ph.v[1] = u[1]; ph.v[2] = (v[2] > 0.f) ? u[2] : -u[2];
            }
            for (int i = 0; i < 3; i++) ph.p[i] += d[i];
            canfocus = false;
            break;
        }
        case 12: case 13: {                                    // line, slit
            const float r = U();
            for (int i = 0; i < 3; i++) ph.p[i] += r * a[i];
            const float len = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
            if (P->srctype == 12) {
                const float ax[3] = {a[0] / len, a[1] / len, a[2] / len};
                if (b[0] > 0.f) {
                    float* v = ph.v;
                    const float dot = v[0] * ax[0] + v[1] * ax[1] + v[2] * ax[2];
                    for (int i = 0; i < 3; i++) v[i] -= dot * ax[i];
                    const float n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                    for (int i = 0; i < 3; i++) v[i] /= n;
                    const float ang = b[0] * (2.f * U() - 1.f), sp = std::sin(ang), cp = std::cos(ang);
                    const float cr[3] = {ax[1] * v[2] - ax[2] * v[1], ax[2] * v[0] - ax[0] * v[2], ax[0] * v[1] - ax[1] * v[0]};
                    for (int i = 0; i < 3; i++) v[i] = v[i] * cp + cr[i] * sp;
                } else {
                    for (int i = 0; i < 3; i++) ph.v[i] = ax[i];
                    const float ang = kTWO_PI * U();
                    rotate_to(1.f, 0.f, std::sin(ang), std::cos(ang));
                }
            } else if (b[0] > 0.f || b[1] > 0.f) {
                const float ang = kTWO_PI * U();
                float sp = std::sin(ang), cp = std::cos(ang);
                const float g = std::sqrt(2.f * scatlen());
                cp *= b[0] * g;
                sp *= b[1] * g / len;
                float* v = ph.v;
                const float nv[3] = {a[1] * v[2] - a[2] * v[1], a[2] * v[0] - a[0] * v[2], a[0] * v[1] - a[1] * v[0]};
                cp /= std::sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
                for (int i = 0; i < 3; i++) v[i] += cp * nv[i] + sp * a[i];
                const float n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                for (int i = 0; i < 3; i++) v[i] /= n;
            }
            for (int i = 0; i < 3; i++) origin[i] = P->srcpos[i] + a[i] * 0.5f;
            canfocus = (P->srctype == 13);
            break;
        }
        default:
            break;
        }
        if (std::fabs(ph.w) <= P->minenergy) return false;
        const float f = P->srcdir[3];
        if (canfocus) {
            if (std::isnan(f)) {
                const float phi = kTWO_PI * U(), th = std::acos(2.f * U() - 1.f);
                rotate_to(std::sin(th), std::cos(th), std::sin(phi), std::cos(phi));
            } else if (f < 0.f && std::isinf(f)) {
                const float phi = kTWO_PI * U(), st = std::sqrt(U());
                rotate_to(st, std::sqrt(1.f - st * st), std::sin(phi), std::cos(phi));
            } else if (f != 0.f) {
                const float sg = (f > 0.f) ? 1.f : -1.f;
                for (int i = 0; i < 3; i++) origin[i] += f * ph.v[i];
                for (int i = 0; i < 3; i++) ph.v[i] = sg * (origin[i] - ph.p[i]);
                const float n = std::sqrt(ph.v[0] * ph.v[0] + ph.v[1] * ph.v[1] + ph.v[2] * ph.v[2]);
                for (int i = 0; i < 3; i++) ph.v[i] /= n;
            }
        }
        if (moved) {
            if (ph.p[0] < 0.f || ph.p[1] < 0.f || ph.p[2] < 0.f || ph.p[0] >= C.maxx || ph.p[1] >= C.maxy || ph.p[2] >= C.maxz) {
                ph.mediaid = 0;
            } else {
                ph.idx1d = (uint32_t)((int)std::floor(ph.p[2]) * C.dimxy + (int)std::floor(ph.p[1]) * C.nx + (int)std::floor(ph.p[0]));
                ph.mediaid = P->vol[ph.idx1d];
            }
        }
        return true;
    }

    bool launch(Photon& ph, Tally& T, Rng& rng) {
        // the photon's source, drawn before its launch when every source runs
        // (src/mcx_core.cu:1217-1227)
        ph.src = 1;
        if (C.P->nextra && C.P->srcid != 1) {
            if (C.P->srcid > 1) ph.src = C.P->srcid;
            else ph.src = (int)(rng.next() * 0.9998f * (float)(C.P->nextra + 1)) + 1;
        }
        const OracleProblem* P = srcs ? srcs + (ph.src - 1) : C.P;
        float attempts = 1.f;
        do {
            ph.p[0] = P->srcpos[0]; ph.p[1] = P->srcpos[1]; ph.p[2] = P->srcpos[2]; ph.w = P->srcpos[3];
            ph.v[0] = P->srcdir[0]; ph.v[1] = P->srcdir[1]; ph.v[2] = P->srcdir[2];
            ph.pscat = 0.f; ph.t = 0.f; ph.pathlen = C.minaccumtime;
            ph.idx1d = P->src_idx;
            ph.mediaid = P->src_med;
            if (P->srctype != 0 && !sample_source(ph, rng, P)) {
                // weight at or below minenergy: draw again (bounded here, unlike the reference)
                attempts += 1.f;
                if (attempts > (float)P->maxvoidstep) return false;
                continue;
            }
            ph.rv[0] = 1.f / ph.v[0]; ph.rv[1] = 1.f / ph.v[1]; ph.rv[2] = 1.f / ph.v[2];
            if ((ph.mediaid & kMED_MASK) == 0) {
                int id = skipvoid(C, ph);
                if (id >= 0) {
                    ph.idx1d = (uint32_t)id;
                    ph.mediaid = P->vol[ph.idx1d];
                }
            }
            ph.fd[0] = (short)std::floor(ph.p[0]);
            ph.fd[1] = (short)std::floor(ph.p[1]);
            ph.fd[2] = (short)std::floor(ph.p[2]);
            attempts += 1.f;
            if (attempts > (float)P->maxvoidstep) return false;
        } while ((ph.mediaid & kMED_MASK) == 0 || std::fabs(ph.w) <= P->minenergy);
        ph.mediaid = C.pick(ph.mediaid, rng);
        ph.prop = C.prop_of(ph.mediaid & kMED_MASK, ph.idx1d);
        if (P->mediaformat == 97) {      // the launch voxel's tissue (src/mcx_core.cu:1246-1251, 1679)
            ph.prop = C.svmc_prop(ph);
            ph.testint = true;
        }
        T.e_launch += ph.w;
        T.launches++;
        ph.w0 = ph.w;
        ph.wlaunch = ph.w;
        ph.nscat = kEPS;
        ph.pathlen = 0.f;
        ph.rv[0] = 1.f / ph.v[0]; ph.rv[1] = 1.f / ph.v[1]; ph.rv[2] = 1.f / ph.v[2];
        ph.isdet = (int)(ph.mediaid & kDET_MASK);
        ph.mediaid &= kMED_MASK;
        if (P->savedet) std::memset(ph.ppath, 0, sizeof(float) * C.partialdata);
        return true;
    }

    // Reflection or refraction at a split voxel's plane (reflectray, src/mcx_core.cu:784-830); the
    // normal points along the flight into the tissue entered.  True when the photon is refracted
    // into the background tissue (label 0), where it ends.
    bool reflectray(Photon& ph, float n1, Rng& rng) {
        const float Icos = std::fabs(ph.v[0] * ph.nv[0] + ph.v[1] * ph.nv[1] + ph.v[2] * ph.nv[2]);
        const float n2 = C.prop[ph.sv_isup ? ph.sv_up : ph.sv_lo].n;
        const float tmp0 = n1 * n1, tmp1 = n2 * n2;
        float tmp2 = 1.f - tmp0 / tmp1 * (1.f - Icos * Icos);
        if (tmp2 > 0.f) {
            float Re = tmp0 * Icos * Icos + tmp1 * tmp2;
            tmp2 = std::sqrt(tmp2);
            const float Im = 2.f * n1 * n2 * Icos * tmp2;
            float Rtotal = (Re - Im) / (Re + Im);
            Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
            Rtotal = (Rtotal + (Re - Im) / (Re + Im)) * 0.5f;
            if (rng.next() <= Rtotal) {
                for (int i = 0; i < 3; i++) ph.v[i] += -2.f * Icos * ph.nv[i];
                ph.sv_isup = !ph.sv_isup;
            } else {
                const float q = n1 / n2;
                for (int i = 0; i < 3; i++) {
                    ph.v[i] += -Icos * ph.nv[i];
                    ph.v[i] = tmp2 * ph.nv[i] + q * ph.v[i];
                    ph.nv[i] = -ph.nv[i];
                }
                // MCX tests the flag itself on the upper side (a split voxel's upper label is never 0)
                if ((ph.sv_isup ? 1 : ph.sv_lo) == 0) return true;
                ph.prop = C.prop[ph.sv_isup ? ph.sv_up : ph.sv_lo];
            }
        } else {
            for (int i = 0; i < 3; i++) ph.v[i] += -2.f * Icos * ph.nv[i];
            ph.sv_isup = !ph.sv_isup;
        }
        const float inv = 1.f / std::sqrt(ph.v[0] * ph.v[0] + ph.v[1] * ph.v[1] + ph.v[2] * ph.v[2]);
        for (int i = 0; i < 3; i++) {
            ph.v[i] *= inv;
            ph.rv[i] = 1.f / ph.v[i];
        }
        return false;
    }

    // One photon with its own per-photon stream.
    void run_photon(uint64_t pid, Tally& T) {
        Rng rng;
        seed_photon(rng, C.P->seed, pid);
        run_photon_with(rng, T);
    }

    // One photon from launch to termination (src/mcx_core.cu:1888-2514), drawing from `rng`.
    void run_photon_with(Rng& rng, Tally& T) {
        const OracleProblem* P = C.P;
        Photon ph;
        std::memset(&ph, 0, sizeof(ph));
        ph.fd[3] = -1;
        if (!launch(ph, T, rng)) return;
        const uint32_t flag = P->savedetflag;
        const int save_nscat = P->savedet && (flag & 0x2);
        const int save_ppath = P->savedet && (flag & 0x4);
        const int save_mom = P->savedet && (flag & 0x8);
        const uint32_t M = C.medianum - 1;
        const float n0 = C.prop[0].n;
        const double maxsteps = 1e9;
        const bool svmc = P->mediaformat == 97;

        for (double guard = 0; guard < maxsteps; guard += 1) {
            T.steps++;
            if (ph.pscat <= 0.f) {
                ph.pscat = -std::log(rng.next() + kEPS);
                if (ph.nscat != kEPS) {
                    float cphi = 1.f, sphi = 0.f, stheta, ctheta, tmp0;
                    tmp0 = kTWO_PI * rng.next();
                    sphi = std::sin(tmp0); cphi = std::cos(tmp0);
                    tmp0 = (ph.nscat > (float)P->gscatter) ? 0.f : ph.prop.g;
                    if (std::fabs(tmp0) > kEPS) {
                        const float g = ph.prop.g;
                        tmp0 = (1.f - g * g) / (1.f - g + 2.f * g * rng.next());
                        tmp0 *= tmp0;
                        tmp0 = (1.f + g * g - tmp0) / (2.f * g);
                        tmp0 = std::fmax(-1.f, std::fmin(1.f, tmp0));
                        float theta = std::acos(tmp0);
                        stheta = std::sin(theta);
                        ctheta = tmp0;
                    } else {
                        float theta = std::acos(2.f * rng.next() - 1.f);
                        stheta = std::sin(theta); ctheta = std::cos(theta);
                    }
                    if (save_nscat) ph.ppath[ph.mediaid - 1] += 1.f;
                    if (save_mom) ph.ppath[M * (save_nscat + save_ppath) + ph.mediaid - 1] += 1.f - ctheta;
                    rotatevector(ph.v, stheta, ctheta, sphi, cphi);
                    ph.nscat += 1.f;
                    ph.rv[0] = 1.f / ph.v[0]; ph.rv[1] = 1.f / ph.v[1]; ph.rv[2] = 1.f / ph.v[2];
                    T.scatters++;
                }
                ph.nscat = (float)(int)ph.nscat;
            }

            float n1 = ph.prop.n;
            if (!svmc) ph.prop = C.prop_of(ph.mediaid, ph.idx1d);

            float len = hitgrid(ph.p, ph.v, ph.rv, ph.fd);
            float musp = ph.prop.mus * ((ph.nscat + 1.f > (float)P->gscatter) ? (1.f - ph.prop.g) : 1.f);
            float slen = len * musp;
            slen = std::fmin(slen, ph.pscat);
            len = (ph.prop.mus == 0.f) ? len : (slen / musp);

            // the flight stops on a split voxel's plane (ray_plane_intersect, src/mcx_core.cu:747-772)
            bool hit = false;
            if (svmc && ph.sv_split && ph.testint) {
                const float vn = ph.v[0] * ph.nv[0] + ph.v[1] * ph.nv[1] + ph.v[2] * ph.nv[2];
                if (vn > 0.f) {
                    float d0 = 0.f, d1 = 0.f;
                    for (int i = 0; i < 3; i++) {
                        d0 += (ph.p[i] - ph.rp[i]) * ph.nv[i];
                        d1 += (ph.p[i] + len * ph.v[i] - ph.rp[i]) * ph.nv[i];
                    }
                    if (!(d0 * d1 > 0.f)) {
                        const float len0 = len * d0 / (d0 - d1);
                        len = (len0 > 0.f) ? len0 : len;
                        slen = len * ph.prop.mus * ((ph.nscat + 1.f > (float)P->gscatter) ? (1.f - ph.prop.g) : 1.f);
                        hit = true;
                    }
                }
            }

            ph.p[0] += len * ph.v[0]; ph.p[1] += len * ph.v[1]; ph.p[2] += len * ph.v[2];
            const bool stay = (slen == ph.pscat) || hit;
            if (ph.fd[3] == 0) ph.fd[0] += stay ? 0 : (ph.v[0] > 0.f ? 1 : -1);
            if (ph.fd[3] == 1) ph.fd[1] += stay ? 0 : (ph.v[1] > 0.f ? 1 : -1);
            if (ph.fd[3] == 2) ph.fd[2] += stay ? 0 : (ph.v[2] > 0.f ? 1 : -1);

            ph.w *= std::exp(-ph.prop.mua * len);
            ph.pscat -= slen;
            ph.t += len * ph.prop.n * C.oneoverc0;
            ph.pathlen += len;
            if (save_ppath) ph.ppath[M * save_nscat + ph.mediaid - 1] += len;

            uint32_t mediaidold = ph.mediaid | ((uint32_t)ph.isdet & kDET_MASK);
            uint32_t idx1dold = ph.idx1d;
            ph.idx1d = vidx(C, ph.fd);
            uint32_t isdet;
            if (!inside(C, ph.fd)) {
                ph.mediaid = 0;
                ph.idx1d = (ph.fd[0] < 0 || ph.fd[1] < 0 || ph.fd[2] < 0) ? kOUT_MIN : kOUT_MAX;
                isdet = (uint8_t)P->bc[(ph.idx1d == kOUT_MAX) * 3 + ph.fd[3]];
            } else {
                uint32_t m = C.pick(P->vol[ph.idx1d], rng);
                isdet = m & kDET_MASK;
                ph.mediaid = m & kMED_MASK;
            }
            ph.isdet = (int)isdet;

            if ((ph.idx1d != idx1dold || hit) && mediaidold) {
                bool rec = false;
                if (P->save2pt && ph.t >= C.twin0 && ph.t < C.twin1) {
                    int tshift = (int)std::floor((ph.t - C.twin0) * C.Rtstep);
                    if (tshift > (int)C.maxgate - 1) tshift = (int)C.maxgate - 1;
                    if (P->nextra && P->srcid < 0) tshift += (ph.src - 1) * (int)C.maxgate;   // 2225-2227
                    float weight = 0.f;
                    if (P->outputtype == 2) weight = ph.w0 - ph.w;                     // energy
                    else if (P->outputtype == 0 || P->outputtype == 1)                 // flux / fluence
                        weight = (ph.prop.mua < kEPS) ? (ph.w0 * ph.pathlen) : (ph.w0 - ph.w) / ph.prop.mua;
                    else if (P->outputtype == 7) weight = ph.w0 * ph.pathlen;          // L
                    if (std::fabs(weight) > 0.f) {
                        deposit(idx1dold, tshift, (double)weight);
                        T.deposits++;
                        rec = true;
                    }
                }
                if (rec) T.e_absdep += (double)ph.w0 - (double)ph.w;
                else T.e_absother += (double)ph.w0 - (double)ph.w;
                ph.w0 = ph.w;
                ph.pathlen = 0.f;
            } else {
                ph.mediaid = mediaidold & kMED_MASK;   // same voxel: the label is unchanged
            }
            const uint32_t med = ph.mediaid;
            const int bcf = (int)(isdet & 0xF);

            // split voxels: a new voxel's tissue at the new position; across the plane, the other
            // tissue (src/mcx_core.cu:2295-2303)
            if (svmc) {
                if (ph.idx1d != idx1dold) {
                    ph.prop = C.svmc_prop(ph);
                    ph.testint = true;
                } else if (hit) {
                    for (int i = 0; i < 3; i++) ph.nv[i] = -ph.nv[i];
                    ph.sv_isup = !ph.sv_isup;
                    ph.testint = false;
                }
            }

            // termination: exit to a 0 voxel without reflection, into a split voxel's background
            // tissue without reflection, or beyond the time window
            if ((med == 0 && ((!C.isreflect || (C.isreflect && n1 == n0)) ||
                              ((bcf == BC_UNKNOWN && !P->isreflect) || bcf == BC_ABSORB || bcf == BC_CYCLIC)) && bcf != BC_MIRROR) ||
                (svmc && (ph.idx1d != idx1dold || hit) && !ph.sv_isup && !ph.sv_lo && (!C.isreflect || n1 == n0)) ||
                ph.t > C.twin1) {
                if (isdet == BC_CYCLIC) {
                    float* pp = ph.p;
                    const float mx[3] = {C.maxx, C.maxy, C.maxz};
                    int a = ph.fd[3];
                    pp[a] = nextafter_mcx(std::round(pp[a] + ((ph.idx1d == kOUT_MIN) ? mx[a] : -mx[a])),
                                          (ph.v[a] > 0.f) - (ph.v[a] < 0.f), (float)P->maxvoidstep);
                    ph.fd[a] = (short)std::floor(pp[a]);
                    if (inside(C, ph.fd)) {
                        ph.idx1d = vidx(C, ph.fd);
                        uint32_t m = C.pick(P->vol[ph.idx1d], rng);
                        ph.isdet = (int)(m & kDET_MASK);
                        ph.mediaid = m & kMED_MASK;
                        continue;
                    }
                }
                uint32_t detflag = (((ph.idx1d == kOUT_MAX && P->bc[9 + ph.fd[3]]) || (ph.idx1d == kOUT_MIN && P->bc[6 + ph.fd[3]]))
                                    ? kOUT_MIN : (mediaidold & kDET_MASK));
                ph.mediaid = med;
                terminate(ph, detflag, T);
                T.photons++;
                return;
            }

            // Russian roulette (src/mcx_core.cu:2357-2378)
            if (std::fabs(ph.w) < P->minenergy) {
                if (rng.next() * 10.f <= 1.f) {
                    ph.w *= 10.f;
                } else {
                    ph.mediaid = med;
                    terminate(ph, mediaidold & kDET_MASK, T);
                    T.photons++;
                    return;
                }
            }

            if (svmc && !C.isreflect) {
                ph.prop = C.prop[ph.sv_isup ? ph.sv_up : ph.sv_lo];   // src/mcx_core.cu:2504-2507
            } else if (svmc && hit) {
                // Fresnel at the plane (src/mcx_core.cu:2386-2404): the normal turned back along the flight
                if (C.prop[ph.sv_lo].n != C.prop[ph.sv_up].n) {
                    for (int i = 0; i < 3; i++) ph.nv[i] = -ph.nv[i];
                    if (reflectray(ph, n1, rng)) {      // out into the background tissue
                        terminate(ph, mediaidold & kDET_MASK, T);
                        T.photons++;
                        return;
                    }
                } else {
                    ph.prop = C.prop[ph.sv_isup ? ph.sv_up : ph.sv_lo];
                }
            } else if (C.isreflect) {
                if (!svmc) ph.prop = C.prop_of(med, ph.idx1d);
                if (((med && P->isreflect) ||
                     (med == 0 && ((bcf == BC_UNKNOWN && P->isreflect) || bcf == BC_REFLECT || bcf == BC_MIRROR))) &&
                    (bcf == BC_MIRROR || n1 != ph.prop.n)) {
                    float Rtotal = 1.f;
                    float tmp0 = n1 * n1, tmp1 = ph.prop.n * ph.prop.n;
                    int a = ph.fd[3];
                    float cphi = std::fabs(ph.v[a]);
                    float sphi = 1.f - cphi * cphi;
                    float c2 = 1.f - tmp0 / tmp1 * sphi;
                    if (c2 > 0.f && bcf != BC_MIRROR) {
                        float ctheta = tmp0 * cphi * cphi + tmp1 * c2;
                        float stheta = 2.f * n1 * ph.prop.n * cphi * std::sqrt(c2);
                        Rtotal = (ctheta - stheta) / (ctheta + stheta);
                        ctheta = tmp1 * cphi * cphi + tmp0 * c2;
                        Rtotal = (Rtotal + (ctheta - stheta) / (ctheta + stheta)) * 0.5f;
                    }
                    if (Rtotal < 1.f && !(med == 0 && bcf == BC_MIRROR) && rng.next() > Rtotal) {
                        transmit(ph.v, n1, ph.prop.n, a);
                        if (med == 0 || (svmc && (ph.sv_isup ? ph.sv_up : ph.sv_lo) == 0)) {
                            uint32_t detflag = (((ph.idx1d == kOUT_MAX && P->bc[9 + a]) || (ph.idx1d == kOUT_MIN && P->bc[6 + a]))
                                                ? kOUT_MIN : (mediaidold & kDET_MASK));
                            ph.mediaid = 0;
                            terminate(ph, detflag, T);
                            T.photons++;
                            return;
                        }
                        ph.rv[0] = 1.f / ph.v[0]; ph.rv[1] = 1.f / ph.v[1]; ph.rv[2] = 1.f / ph.v[2];
                    } else {
                        ph.v[a] = -ph.v[a];
                        ph.rv[0] = 1.f / ph.v[0]; ph.rv[1] = 1.f / ph.v[1]; ph.rv[2] = 1.f / ph.v[2];
                        ph.p[a] = nextafter_mcx(std::nearbyint(ph.p[a]), (ph.v[a] > 0.f) - (ph.v[a] < 0.f), (float)P->maxvoidstep);
                        ph.fd[a] = (short)std::floor(ph.p[a]);
                        ph.idx1d = idx1dold;
                        ph.mediaid = C.pick(P->vol[ph.idx1d], rng) & kMED_MASK;
                        if (!svmc) {
                            ph.prop = C.prop_of(ph.mediaid, ph.idx1d);
                        } else {
                            // back in the voxel it left: its tissue at the reflected position; reflected
                            // into a split voxel's background tissue, the photon ends
                            // (src/mcx_core.cu:2474-2490)
                            ph.prop = C.svmc_prop(ph);
                            if ((ph.sv_isup ? ph.sv_up : ph.sv_lo) == 0) {
                                terminate(ph, mediaidold & kDET_MASK, T);
                                T.photons++;
                                return;
                            }
                        }
                    }
                } else if (!svmc) {
                    ph.prop = C.prop_of(mediaidold & kMED_MASK, idx1dold);
                }
            }
        }
        // unreachable for physical inputs; counted as escaped so the balance still closes
        terminate(ph, 0, T);
        T.photons++;
    }
};

}  // namespace

extern "C" {

int oracle_version(void) { return 1; }

// src/mcx_core.cu:1731-1742 with the host seeding of src/mcx_core.cu:3062-3066: the
// generator is seeded with four 32-bit words and emits n uniform floats.
void oracle_rng_kat(const uint32_t seeds[4], float* out, int n) {
    Rng r;
    r.s[0] = ((uint64_t)seeds[0] << 32) | seeds[1];
    r.s[1] = ((uint64_t)seeds[2] << 32) | seeds[3];
    for (int i = 0; i < n; i++) out[i] = r.next();
}

// Per-photon seeded stream, identical to the GB300 engine's: n floats of photon `pid`.
void oracle_photon_stream(uint64_t seed, uint64_t pid, float* out, int n) {
    Rng r;
    seed_photon(r, seed, pid);
    for (int i = 0; i < n; i++) out[i] = r.next();
}

int oracle_run(const OracleProblem* P, OracleResult* R) {
    if (!P || !R || !P->vol || !P->prop || P->medianum < 1 || P->medianum > 128) return -1;
    if (!R->field && P->save2pt) return -2;
    Ctx C;
    C.P = P;
    C.nx = P->dim[0]; C.ny = P->dim[1]; C.nz = P->dim[2];
    C.dimxy = C.nx * C.ny; C.dimxyz = C.dimxy * C.nz;
    C.maxx = (float)C.nx; C.maxy = (float)C.ny; C.maxz = (float)C.nz;
    C.oneoverc0 = kR_C0 * P->unitinmm;
    C.minaccumtime = kR_C0 * P->unitinmm;
    C.Rtstep = 1.f / P->tstep;
    C.twin0 = P->twin0;
    C.twin1 = P->twin1;
    C.maxgate = P->maxgate;
    C.medianum = P->medianum;
    C.detnum = P->detnum;
    uint32_t flag = P->savedetflag;
    C.partialdata = (P->medianum - 1) * (((flag >> 1) & 1) + ((flag >> 2) & 1) + ((flag >> 3) & 1));
    C.reclen = C.partialdata + (flag & 1) + 3 * (((flag >> 4) & 1) + ((flag >> 5) & 1)) + ((flag >> 6) & 1);
    C.isreflect = P->isreflect;
    for (int i = 0; i < 6; i++)
        if (P->bc[i] == BC_REFLECT || P->bc[i] == BC_MIRROR) C.isreflect = 1;
    std::vector<Prop> props(P->medianum);
    for (uint32_t i = 0; i < P->medianum; i++) props[i] = {P->prop[4 * i], P->prop[4 * i + 1], P->prop[4 * i + 2], P->prop[4 * i + 3]};
    C.prop = props.data();

    // the extra sources as problems of their own: position, direction, parameters and, for
    // point sources, the launch voxel and its label (src/mcx_utils.c:1679-1692, 1748-1756)
    std::vector<OracleProblem> srcs(1 + (P->extrasrc ? P->nextra : 0), *P);
    for (uint32_t k = 1; k < srcs.size(); k++) {
        OracleProblem& S = srcs[k];
        const float* x = P->extrasrc + 16 * (k - 1);
        std::memcpy(S.srcpos, x, 4 * sizeof(float));
        std::memcpy(S.srcdir, x + 4, 4 * sizeof(float));
        std::memcpy(S.srcparam1, x + 8, 4 * sizeof(float));
        std::memcpy(S.srcparam2, x + 12, 4 * sizeof(float));
        if (S.srcpos[3] == 0.f) S.srcpos[3] = 1.f;
        const float nd = std::sqrt(S.srcdir[0] * S.srcdir[0] + S.srcdir[1] * S.srcdir[1] + S.srcdir[2] * S.srcdir[2]);
        if (nd > 0.f)
            for (int i = 0; i < 3; i++) S.srcdir[i] /= nd;
        S.src_idx = 0;
        S.src_med = 0;
        if (S.srcpos[0] >= 0.f && S.srcpos[1] >= 0.f && S.srcpos[2] >= 0.f && S.srcpos[0] < C.maxx &&
            S.srcpos[1] < C.maxy && S.srcpos[2] < C.maxz) {
            S.src_idx = (uint32_t)((int)std::floor(S.srcpos[2]) * C.dimxy + (int)std::floor(S.srcpos[1]) * C.nx +
                                   (int)std::floor(S.srcpos[0]));
            S.src_med = P->vol[S.src_idx] & kMED_MASK;
        }
    }

    std::atomic<uint64_t> slot(0);
    Runner run;
    run.C = C;
    run.R = R;
    run.detslot = &slot;
    run.srcs = srcs.data();

    int nthreads = P->nthreads > 0 ? P->nthreads : 1;
    std::vector<Tally> tallies(nthreads);
    // MCX's seeds: srand(seed) then four (rand()<<16)|(rand()<<1)|(rand()>>14) words per stream
    // (src/mcx_core.cu:3247-3251, 3381-3387), drawn in stream order
    std::vector<uint32_t> words;
    if (P->seed_mode == 1) {
        if (P->mcx_threads == 0) return -3;
        words.resize((size_t)P->mcx_threads * 4);
        srand((unsigned)P->seed);
        for (auto& wd : words) {
            const unsigned a = (unsigned)rand(), b = (unsigned)rand(), c = (unsigned)rand();
            wd = (a << 16) | (b << 1) | (c >> 14);
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    const int64_t N = (int64_t)P->nphoton;
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        Tally& T = tallies[tid];
        if (P->seed_mode == 1) {
            // MCX's static partition: stream i runs threadphoton (+1 for i < oddphotons) photons
            const int64_t nthr = (int64_t)words.size() / 4;
            const int64_t per = N / nthr, odd = N - per * nthr;
#pragma omp for schedule(dynamic, 64)
            for (int64_t i = 0; i < nthr; i++) {
                Rng rng;
                rng.s[0] = ((uint64_t)words[4 * i] << 32) | words[4 * i + 1];
                rng.s[1] = ((uint64_t)words[4 * i + 2] << 32) | words[4 * i + 3];
                const int64_t n = per + (i < odd ? 1 : 0);
                for (int64_t k = 0; k < n; k++) run.run_photon_with(rng, T);
            }
        } else {
#pragma omp for schedule(dynamic, 256)
            for (int64_t i = 0; i < N; i++) run.run_photon(P->photon_offset + (uint64_t)i, T);
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    Tally S;
    for (auto& T : tallies) {
        S.e_launch += T.e_launch; S.e_escape += T.e_escape; S.e_detect += T.e_detect;
        S.e_absdep += T.e_absdep; S.e_absother += T.e_absother;
        S.steps += T.steps; S.scatters += T.scatters; S.deposits += T.deposits;
        S.launches += T.launches; S.detected += T.detected; S.photons += T.photons;
    }
    R->e_launch = S.e_launch; R->e_escape = S.e_escape; R->e_detect = S.e_detect;
    R->e_absdep = S.e_absdep; R->e_absother = S.e_absother;
    R->n_steps = S.steps; R->n_scatter = S.scatters; R->n_deposit = S.deposits;
    R->n_launch = S.launches; R->n_detected = S.detected; R->n_photon = S.photons;
    R->n_saved = slot.load() < P->maxdetphoton ? slot.load() : P->maxdetphoton;
    R->reclen = C.reclen;
    R->seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

}  // extern "C"
