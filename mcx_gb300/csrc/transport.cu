// transport.cu -- the GB300 photon-transport kernel (sm_103a).
//
// Algorithm: MCX's voxel Monte Carlo (src/mcx_core.cu:1767-2528, label media) with its photon
// launch (src/mcx_core.cu:1089-1717, every source shape), one photon per thread, re-organised
// for Blackwell:
//   * persistent CTAs (grid = SMs x resident CTAs) whose warps refill dead lanes from a
//     warp-private pool of photon indices, topped up with one global atomic per `chunk`
//     photons -- no lane waits for a slow photon of another lane to finish a static quota;
//   * every photon owns an xorshift128+ state in registers, seeded from (seed, photon index)
//     so results do not depend on grid shape or scheduling (or MCX's own per-thread streams);
//   * labels are one byte per voxel (bit 7 = detector mask) read through the read-only
//     path; the (mua, mus, g, n) table lives in shared memory because lanes index it with
//     divergent labels;
//   * fluence deposits inside a per-CTA voxel x gate box over the launch point go to an exact
//     32-bit fixed-point shared-memory tile and reach L2 once per CTA; the rest are
//     fire-and-forget FP32 reductions;
//   * three variants per flag set: pencil beam (mode 0), other source shapes sampled per
//     photon (1), replay / seed saving / replay outputs (2), so each carries only its state;
//   * FP64 is used only for the energy tallies.
// Semantics that must match the reference step for step are annotated with its file:line.

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdint>
#include "transport.cuh"

namespace mcxg {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// xorshift128+ step, float from the low 32 bits (src/mcx_rand_xorshift128p.cu:56-72).
__device__ __forceinline__ float rng_next(unsigned long long& a, unsigned long long& b) {
    unsigned long long s1 = a;
    const unsigned long long s0 = b;
    a = s0;
    s1 ^= s1 << 23;
    b = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
    const unsigned lo = (unsigned)(b + s0);
    return __uint_as_float(0x3F800000u | (lo >> 9)) - 1.0f;
}

// One xorshift128+ step giving three uniforms in [0, 1) with 21-bit resolution, from bits 43-63,
// 22-42 and 1-21 of the 64-bit output: the random numbers of one scattering event for the
// per-photon streams, which need not follow MCX's draw-by-draw consumption.
__device__ __forceinline__ void rng_next3(unsigned long long& a, unsigned long long& b, float& f0, float& f1,
                                          float& f2) {
    unsigned long long s1 = a;
    const unsigned long long s0 = b;
    a = s0;
    s1 ^= s1 << 23;
    b = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
    const unsigned long long r = b + s0;
    f0 = __uint_as_float(0x3F800000u | (((unsigned)(r >> 32) >> 9) & 0x7FFFFCu)) - 1.0f;
    f1 = __uint_as_float(0x3F800000u | ((unsigned)(r >> 20) & 0x7FFFFCu)) - 1.0f;
    f2 = __uint_as_float(0x3F800000u | (((unsigned)r << 1) & 0x7FFFFCu)) - 1.0f;
}

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long& x) {
    unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-photon stream: identical to oracle/mcx_oracle.cpp seed_photon().
__device__ __forceinline__ void seed_photon(unsigned long long seed, unsigned long long pid,
                                            unsigned long long& a, unsigned long long& b) {
    unsigned long long x = seed * 0xD1B54A32D192ED03ull + pid;
    a = splitmix64(x);
    b = splitmix64(x);
    if ((a | b) == 0ull) b = 1ull;
}

// src/mcx_core.cu:470-478: move a coordinate one ulp towards `dir` after an offset that keeps
// it positive.
__device__ __forceinline__ float nextafter_mcx(float a, int dir, float offset) {
    unsigned i = __float_as_uint(a + offset);
    i += (unsigned)dir ^ (i & 0x80000000u);
    return __uint_as_float(i) - offset;
}

// src/mcx_core.cu:1011-1031
__device__ __forceinline__ void rotate(float& vx, float& vy, float& vz, float st, float ct, float sp, float cp) {
    float nx, ny, nz;
    if (vz > -1.f + kEPS && vz < 1.f - kEPS) {
        const float t0 = 1.f - vz * vz;
        const float t1 = st * rsqrtf(t0);
        nx = t1 * (vx * vz * cp - vy * sp) + vx * ct;
        ny = t1 * (vy * vz * cp + vx * sp) + vy * ct;
        nz = -t1 * t0 * cp + vz * ct;
    } else {
        nx = st * cp;
        ny = st * sp;
        nz = (vz > 0.f) ? ct : -ct;
    }
    const float r = rsqrtf(nx * nx + ny * ny + nz * nz);
    vx = nx * r; vy = ny * r; vz = nz * r;
}

// src/mcx_core.cu:523-537: refraction applied to the axis normal to the face, renormalised.
__device__ __forceinline__ void transmit(float& vx, float& vy, float& vz, float n1, float n2, int axis) {
    const float r = __fdividef(n1, n2);
    vx *= r; vy *= r; vz *= r;
    if (axis == 0) {
        const float s = vy * vy + vz * vz;
        vx = (s < 1.f) ? sqrtf(1.f - s) * (float)((vx > 0.f) - (vx < 0.f)) : 0.f;
    } else if (axis == 1) {
        const float s = vx * vx + vz * vz;
        vy = (s < 1.f) ? sqrtf(1.f - s) * (float)((vy > 0.f) - (vy < 0.f)) : 0.f;
    } else {
        const float s = vx * vx + vy * vy;
        vz = (s < 1.f) ? sqrtf(1.f - s) * (float)((vz > 0.f) - (vz < 0.f)) : 0.f;
    }
    const float k = rsqrtf(vx * vx + vy * vy + vz * vz);
    vx *= k; vy *= k; vz *= k;
}

// src/mcx_core.cu:258-270
__device__ int find_detector(const KParams& P, float px, float py, float pz) {
    for (int i = 0; i < P.ndet; i++) {
        const float4 d = P.detpos[i];
        if ((d.x - px) * (d.x - px) + (d.y - py) * (d.y - py) + (d.z - pz) * (d.z - pz) < d.w * d.w)
            return (d.w < 0.f) ? 0 : i + 1;
    }
    return 0;
}

// ---- sources other than the pencil beam -------------------------------------------------------
// A launched photon: position, weight, direction, time (grid units), voxel and its label byte.
struct Launch {
    float px, py, pz, w, vx, vy, vz, t;
    unsigned idx, label;
    unsigned pix;               // photon sharing: the pattern pixel the photon started from
    int ix, iy, iz;             // integer coordinates of voxel idx (the position may sit on its face)
};

// src/mcx_core.cu:552-570 (reflectcoeff): unpolarised Fresnel reflectance at a face normal to
// `axis` going from index n1 to n2.
__device__ __forceinline__ float reflect_coeff(float vx, float vy, float vz, float n1, float n2, int axis) {
    const float Icos = fabsf(axis == 0 ? vx : (axis == 1 ? vy : vz));
    const float a = n1 * n1, b = n2 * n2;
    float c = 1.f - __fdividef(a, b) * (1.f - Icos * Icos);
    if (c <= 0.f) return 1.f;
    float Re = a * Icos * Icos + b * c;
    c = sqrtf(c);
    const float Im = 2.f * n1 * n2 * Icos * c;
    float R = __fdividef(Re - Im, Re + Im);
    Re = b * Icos * Icos + a * c * c;
    return (R + __fdividef(Re - Im, Re + Im)) * 0.5f;
}

// Voxel contents: a byte label (bit 7 detector mask, bits 0-6 medium) or, for the per-voxel media
// formats, MCX's 32-bit word (bit 31 detector mask, bits 0-30 the encoded properties; 0 = void).
template <bool WORDS>
__device__ __forceinline__ unsigned voxel_load(const KParams& P, unsigned idx) {
    if (WORDS) return __ldg(P.words + idx);
    return (unsigned)__ldg(P.labels + idx);
}
template <bool WORDS>
__device__ __forceinline__ unsigned voxel_med(unsigned v) { return WORDS ? (v & kMED_MASK) : (v & kLabelMask); }
template <bool WORDS>
__device__ __forceinline__ bool voxel_det(unsigned v) { return WORDS ? (v >> 31) != 0u : (v & kLabelDet) != 0u; }

__device__ __forceinline__ float half_bits(unsigned h) { return __half2float(__ushort_as_half((unsigned short)h)); }

// MEDIA_2LABEL_MIX (src/mcx_core.cu:649-666): a voxel word [fraction (15 bits)][label 1][label 0]
// is tissue 1 with probability fraction / 32767, else tissue 0, drawn once when the photon enters
// the voxel (MCX draws at its first step there and keeps the choice for the voxel).  Returns the
// word with the chosen label in place and the detector bit kept; other formats pass through.
template <bool WORDS>
__device__ __forceinline__ unsigned voxel_pick(const KParams& P, unsigned lab, unsigned long long& r0,
                                               unsigned long long& r1) {
    if (!WORDS || P.mediaformat != kMedia2LabelMix) return lab;
    const unsigned frac = (lab >> 16) & 0x7FFFu;
    unsigned c = lab & 0xFFu;
    if (frac > 0u && rng_next(r0, r1) * 32767.f < (float)frac) c = (lab >> 8) & 0xFFu;
    return (lab & kDET_MASK) | c;
}

// Optical properties (mua, mus, g, n) of a voxel's medium value m (src/mcx_core.cu:582-730):
// the table row for labels; decoded from the word for the per-voxel formats, whose missing
// fields come from table rows 1 and 2 (MEDIA_LABEL_HALF: from the row of the word's label;
// MEDIA_ASGN_F2H stores all four, two in a second word per voxel).  `idx` is the voxel's index.  A void or outside voxel (m = 0) takes row 0 in every
// format; MCX decodes it like any word, which for MEDIA_ASGN_BYTE gives the outside row 2's n
// and mus, so photons there scatter outside the volume.
template <bool WORDS>
__device__ __forceinline__ float4 props_of(const KParams& P, const float4* tab, unsigned m, unsigned idx) {
    if (!WORDS || m == 0u) return tab[m];     // void and outside: row 1 of prop, as for labels
    if (P.mediaformat == kMedia2LabelMix) return tab[m & 0xFFu];     // resolved to one label (voxel_pick)
    if (P.mediaformat == kMedia2LabelSplit) return tab[m >> 24];     // the lower label (split_voxel_at decides)
    if (P.mediaformat == kMediaAsgnF2H) {
        // [n][g] halves in the voxel's second word, [mus][mua] in the first (src/mcx_core.cu:628-647)
        const unsigned m2 = __ldg(P.words2 + idx);
        return make_float4(fabsf(half_bits(m & 0xFFFFu)), fabsf(half_bits(m >> 16)), fabsf(half_bits(m2 & 0xFFFFu)),
                           fabsf(half_bits(m2 >> 16)));
    }
    if (P.mediaformat == kMediaLabelHalf) {
        // [half value][2-bit field | 14-bit label]: the label's row with one field replaced
        float4 r = tab[m & 0x3FFFu];
        const float v = fabsf(half_bits(m >> 16));
        const unsigned f = (m >> 14) & 3u;
        if (f == 0u) r.x = v;
        else if (f == 1u) r.y = v;
        else if (f == 2u) r.z = v;
        else r.w = v;
        return r;
    }
    const float4 r1 = tab[1];
    const float n = r1.w;
    if (P.mediaformat == kMediaMuaFloat) return make_float4(__uint_as_float(m), r1.y, r1.z, n);
    if (P.mediaformat == kMediaAsF2H || P.mediaformat == kMediaAsHalf)
        return make_float4(fabsf(half_bits(m & 0xFFFFu)), fabsf(half_bits(m >> 16)), r1.z, n);
    const float4 r2 = tab[2];
    if (P.mediaformat == kMediaAsgnByte) {
        return make_float4((m & 0xFFu) * (1.f / 255.f) * (r2.x - r1.x) + r1.x,
                           ((m >> 8) & 0xFFu) * (1.f / 255.f) * (r2.y - r1.y) + r1.y,
                           ((m >> 16) & 0xFFu) * (1.f / 255.f) * (r2.z - r1.z) + r1.z,
                           (m >> 24) * (1.f / 127.f) * (r2.w - r1.w) + r1.w);
    }
    // kMediaAsShort
    return make_float4((m & 0xFFFFu) * (1.f / 65535.f) * (r2.x - r1.x) + r1.x,
                       (m >> 16) * (1.f / 65535.f) * (r2.y - r1.y) + r1.y, r1.z, n);
}

__device__ __forceinline__ bool in_grid(const KParams& P, int x, int y, int z) {
    return (unsigned)x < (unsigned)P.nx && (unsigned)y < (unsigned)P.ny && (unsigned)z < (unsigned)P.nz;
}

// Split voxel (MEDIA_2LABEL_SPLIT, SVMC; updateproperty, src/mcx_core.cu:688-730).  Two words per
// voxel: the first [lower label][upper label][plane point x][plane point y], the second [plane
// point z][normal x][normal y][normal z], bytes scaled to [0, 1] (point, within the voxel) and
// [-1, 1] (normal).  A voxel with upper label 0 is plain (its lower label); in a split one the
// photon is in the upper tissue when it lies on the side the normal points away from, and the
// stored normal then points to the other side (outward from the photon's tissue).
struct SplitVoxel {
    int lo, up;
    bool split, isup;
    float rx, ry, rz, nx, ny, nz;
    __device__ __forceinline__ int tissue() const { return isup ? up : lo; }
};

__device__ __forceinline__ void split_voxel_at(const KParams& P, unsigned vidx, float fx, float fy, float fz, float px,
                                               float py, float pz, SplitVoxel& sv) {
    const unsigned wa = __ldg(P.words + vidx) & kMED_MASK, wb = __ldg(P.words2 + vidx);
    sv.lo = (int)(wa >> 24);
    sv.up = (int)((wa >> 16) & 0xFFu);
    sv.isup = false;
    float nx = ((wb >> 16) & 0xFFu) * (2.f / 255.f) - 1.f, ny = ((wb >> 8) & 0xFFu) * (2.f / 255.f) - 1.f,
          nz = (wb & 0xFFu) * (2.f / 255.f) - 1.f;
    const float nn = nx * nx + ny * ny + nz * nz;
    sv.split = sv.up != 0 && nn > 0.f;
    if (sv.split) {
        sv.rx = ((wa >> 8) & 0xFFu) * (1.f / 255.f) + fx;
        sv.ry = (wa & 0xFFu) * (1.f / 255.f) + fy;
        sv.rz = (wb >> 24) * (1.f / 255.f) + fz;
        const float inv = rsqrtf(nn);
        nx *= inv; ny *= inv; nz *= inv;
        if ((sv.rx - px) * nx + (sv.ry - py) * ny + (sv.rz - pz) * nz < 0.f) {
            sv.isup = true;
            nx = -nx; ny = -ny; nz = -nz;
        }
        sv.nx = nx; sv.ny = ny; sv.nz = nz;
    }
}

// src/mcx_core.cu:866-956 (skipvoid): march a photon launched outside the volume or in a 0 voxel
// in unit steps until it is inside a non-zero voxel, back up one step and find the exact entry
// face with voxel-to-voxel steps; optional specular loss and refraction there.  Returns the
// entry voxel, or -1 when the photon misses the volume.
template <bool WORDS>
__device__ int skip_void(const KParams& P, Launch& L) {
    const float rvx = __fdividef(1.f, L.vx), rvy = __fdividef(1.f, L.vy), rvz = __fdividef(1.f, L.vz);
    int fx = (int)floorf(L.px), fy = (int)floorf(L.py), fz = (int)floorf(L.pz);
    int count = 1;
    while (true) {
        const auto at = [&](int x, int y, int z) {
            return voxel_load<WORDS>(P, (unsigned)z * P.dimxy + (unsigned)y * (unsigned)P.nx + (unsigned)x);
        };
        if (in_grid(P, fx, fy, fz) && voxel_med<WORDS>(at(fx, fy, fz))) {
            L.px -= L.vx; L.py -= L.vy; L.pz -= L.vz;
            fx = (int)floorf(L.px); fy = (int)floorf(L.py); fz = (int)floorf(L.pz);
            L.t -= 1.f;
            int axis = -1;
            for (int k = 0; k <= 4 && !(in_grid(P, fx, fy, fz) && voxel_med<WORDS>(at(fx, fy, fz))); k++) {
                const float hx = fabsf((fx + (L.vx > 0.f ? 1.f : 0.f) - L.px) * rvx);
                const float hy = fabsf((fy + (L.vy > 0.f ? 1.f : 0.f) - L.py) * rvy);
                const float hz = fabsf((fz + (L.vz > 0.f ? 1.f : 0.f) - L.pz) * rvz);
                const float d = fminf(fminf(hx, hy), hz);
                axis = (d == hx) ? 0 : ((d == hy) ? 1 : 2);
                L.t += d;
                L.px += d * L.vx; L.py += d * L.vy; L.pz += d * L.vz;
                if (axis == 0) fx += (L.vx > 0.f) ? 1 : -1;
                else if (axis == 1) fy += (L.vy > 0.f) ? 1 : -1;
                else fz += (L.vz > 0.f) ? 1 : -1;
            }
            if (!in_grid(P, fx, fy, fz)) return -1;
            if (!P.voidtime) L.t = 0.f;
            const unsigned lab = at(fx, fy, fz);
            const unsigned eidx = (unsigned)fz * P.dimxy + (unsigned)fy * (unsigned)P.nx + (unsigned)fx;
            float n2 = props_of<WORDS>(P, P.prop, voxel_med<WORDS>(lab), eidx).w;
            if (P.mediaformat == kMedia2LabelSplit) {
                SplitVoxel sv;
                split_voxel_at(P, eidx, (float)fx, (float)fy, (float)fz, L.px, L.py, L.pz, sv);
                n2 = P.prop[sv.tissue()].w;
            }
            const float n0 = P.prop[0].w;
            if (P.isspecular && axis >= 0 && n2 != n0) {
                L.w *= 1.f - reflect_coeff(L.vx, L.vy, L.vz, n0, n2, axis);
                if (L.w > kEPS) transmit(L.vx, L.vy, L.vz, n0, n2, axis);
            }
            // the entry voxel as the search found it: the position lies on its face, possibly a
            // rounding error outside, so the photon's voxel coordinates are these, not floor(p)
            L.ix = fx; L.iy = fy; L.iz = fz;
            return (int)((unsigned)fz * P.dimxy + (unsigned)fy * (unsigned)P.nx + (unsigned)fx);
        }
        if ((L.px < 0.f && L.vx <= 0.f) || (L.px >= P.d_fnx && L.vx >= 0.f) || (L.py < 0.f && L.vy <= 0.f) ||
            (L.py >= P.d_fny && L.vy >= 0.f) || (L.pz < 0.f && L.vz <= 0.f) || (L.pz >= P.d_fnz && L.vz >= 0.f))
            return -1;
        L.px += L.vx; L.py += L.vy; L.pz += L.vz;
        fx = (int)floorf(L.px); fy = (int)floorf(L.py); fz = (int)floorf(L.pz);
        L.t += 1.f;
        if (count++ > (int)P.maxvoidstep) return -1;
    }
}

// Position shift by r along the azimuth (cphi, sphi) of the plane normal to v (the disk and
// Gaussian branches of src/mcx_core.cu:1372-1420).
__device__ __forceinline__ void offset_normal(Launch& L, float r, float sphi, float cphi) {
    if (L.vz > -1.f + kEPS && L.vz < 1.f - kEPS) {
        const float t0 = 1.f - L.vz * L.vz;
        const float t1 = r * rsqrtf(t0);
        L.px += t1 * (L.vx * L.vz * cphi - L.vy * sphi);
        L.py += t1 * (L.vy * L.vz * cphi + L.vx * sphi);
        L.pz -= t1 * t0 * cphi;
    } else {
        L.px += r * cphi;
        L.py += r * sphi;
    }
}

// One launch of a non-pencil source, drawing from the photon's stream in MCX's order
// (launchnewphoton, src/mcx_core.cu:1236-1672).  Retries a photon that misses the volume up to
// maxvoidstep times; false when every attempt missed.
// Inlined: a call here (tried) forced the loop's live state through the call's stack frame and
// cost the planar deck 21% (143.7 K against 182.7 K photons/ms at 1e8 photons).
template <bool WORDS, bool FULL>
__device__ __forceinline__ bool launch_source(const KParams& P, unsigned long long& r0, unsigned long long& r1, Launch& L,
                                              const float4* __restrict__ alt = nullptr) {
    // the source: the primary one from the parameters, or an extra source's five float4
    // (position, direction, param1, param2, (focus class, focal length)) -- full kernel only
    const bool ALT = FULL && alt != nullptr;
    const float4 p1 = ALT ? alt[2] : P.src_param1, p2 = ALT ? alt[3] : P.src_param2;
    const float4 sp = ALT ? alt[0] : P.src_p, sv = ALT ? alt[1] : P.src_v;
    const int sfocus = ALT ? (int)alt[4].x : P.src_focus;
    const float sfocal = ALT ? alt[4].y : P.src_focal;
    constexpr float kJustBelowOne = 0.9998f;                      // src/mcx_const.h:50
    for (int attempt = 1; attempt <= (int)P.maxvoidstep; attempt++) {
        L.px = sp.x; L.py = sp.y; L.pz = sp.z; L.w = sp.w;
        L.vx = sv.x; L.vy = sv.y; L.vz = sv.z;
        L.t = 0.f;
        float ox = sp.x, oy = sp.y, oz = sp.z;     // focus origin
        bool canfocus = true, located = false;
        switch (P.srctype) {
        case kSrcPlanar: case kSrcPattern: case kSrcPattern3D: case kSrcFourier: case kSrcPencilArray: {
            const float rx = rng_next(r0, r1), ry = rng_next(r0, r1);
            if (P.srctype == kSrcPattern3D) {
                const float rz = rng_next(r0, r1);
                L.px += rx * p1.x; L.py += ry * p1.y; L.pz += rz * p1.z;
                const int nx = (int)p1.x, ny = (int)p1.y;
                const unsigned pix = (int)(rz * kJustBelowOne * p1.z) * ny * nx + (int)(ry * kJustBelowOne * p1.y) * nx +
                                     (int)(rx * kJustBelowOne * p1.x);
                if (P.srcnum > 1) {         // photon sharing: unit weight, the patterns' weights per deposit
                    L.pix = pix;
                    L.w = 1.f;
                } else {
                    L.w = sp.w * __ldg(P.srcpattern + pix);
                }
            } else {
                L.px += rx * p1.x + ry * p2.x; L.py += rx * p1.y + ry * p2.y; L.pz += rx * p1.z + ry * p2.z;
                if (P.srctype == kSrcPattern) {
                    const unsigned pix = (int)(ry * kJustBelowOne * p2.w) * (int)p1.w + (int)(rx * kJustBelowOne * p1.w);
                    if (P.srcnum > 1) {     // photon sharing (src/mcx_core.cu:1288-1296)
                        L.pix = pix;
                        L.w = 1.f;
                    } else {
                        L.w = sp.w * __ldg(P.srcpattern + pix);
                    }
                } else if (P.srctype == kSrcFourier) {
                    L.w = sp.w * (cosf((floorf(p1.w) * rx + floorf(p2.w) * ry + p1.w - floorf(p1.w)) * kTWO_PI) *
                                           (1.f - p2.w + floorf(p2.w)) + 1.f) * 0.5f;
                } else if (P.srctype == kSrcPencilArray) {
                    const float ix = floorf(rx * p1.w) / (p1.w - 1.f), iy = floorf(ry * p2.w) / (p2.w - 1.f);
                    L.px = sp.x + ix * p1.x + iy * p2.x;
                    L.py = sp.y + ix * p1.y + iy * p2.y;
                    L.pz = sp.z + ix * p1.z + iy * p2.z;
                }
            }
            ox += (p1.x + p2.x) * 0.5f; oy += (p1.y + p2.y) * 0.5f; oz += (p1.z + p2.z) * 0.5f;
            break;
        }
        case kSrcFourierX: case kSrcFourierX2D: {
            const float rx = rng_next(r0, r1), ry = rng_next(r0, r1);
            const float s = p1.w * rsqrtf(p1.x * p1.x + p1.y * p1.y + p1.z * p1.z);
            const float v2x = s * (L.vy * p1.z - L.vz * p1.y), v2y = s * (L.vz * p1.x - L.vx * p1.z),
                        v2z = s * (L.vx * p1.y - L.vy * p1.x);
            L.px += rx * p1.x + ry * v2x; L.py += rx * p1.y + ry * v2y; L.pz += rx * p1.z + ry * v2z;
            if (P.srctype == kSrcFourierX2D)
                L.w = sp.w * (sinf((p2.x * rx + p2.z) * kTWO_PI) * sinf((p2.y * ry + p2.w) * kTWO_PI) + 1.f) * 0.5f;
            else
                L.w = sp.w * (cosf((p2.x * rx + p2.y * ry + p2.z) * kTWO_PI) * (1.f - p2.w) + 1.f) * 0.5f;
            ox += (p1.x + v2x) * 0.5f; oy += (p1.y + v2y) * 0.5f; oz += (p1.z + v2z) * 0.5f;
            break;
        }
        case kSrcDisk: case kSrcRing: case kSrcGaussian: {
            float phi;
            if (P.srctype == kSrcRing && (p1.z > 0.f || p1.w > 0.f))
                phi = fabsf(p1.z - p1.w) * rng_next(r0, r1) + fminf(p1.z, p1.w);
            else
                phi = kTWO_PI * rng_next(r0, r1);
            float sphi, cphi;
            sincosf(phi, &sphi, &cphi);
            float r;
            if (P.srctype != kSrcGaussian) {
                r = sqrtf(rng_next(r0, r1) * fabsf(p1.x * p1.x - p1.y * p1.y) + p1.y * p1.y);
            } else if (fabsf(sfocal) < 1e-5f || fabsf(p1.y) < 1e-5f) {
                r = sqrtf(0.5f * -logf(rng_next(r0, r1) + kEPS)) * p1.x;
            } else {
                const float zr = p1.x * p1.x * 3.14159265358979f / p1.y;        // Rayleigh range
                r = sqrtf(0.5f * -logf(rng_next(r0, r1) + kEPS) * (1.f + sfocal * sfocal / (zr * zr))) * p1.x;
            }
            offset_normal(L, r, sphi, cphi);
            break;
        }
        case kSrcCone: case kSrcIsotropic: case kSrcArcsine: {
            float sphi, cphi, st, ct, ang = kTWO_PI * rng_next(r0, r1);
            sincosf(ang, &sphi, &cphi);
            if (P.srctype == kSrcCone) {
                const float c = cosf(p1.x);
                ang = (p1.y > 0.f) ? rng_next(r0, r1) * p1.x : acosf(rng_next(r0, r1) * (1.f - c) + c);
            } else if (P.srctype == kSrcIsotropic) {
                ang = acosf(2.f * rng_next(r0, r1) - 1.f);
            } else {
                ang = 3.14159265358979f * rng_next(r0, r1);
            }
            sincosf(ang, &st, &ct);
            rotate(L.vx, L.vy, L.vz, st, ct, sphi, cphi);
            canfocus = false;
            located = true;
            break;
        }
        case kSrcZGaussian: {
            float sphi, cphi, st, ct, ang = kTWO_PI * rng_next(r0, r1);
            sincosf(ang, &sphi, &cphi);
            ang = sqrtf(2.f * -logf(rng_next(r0, r1) + kEPS));
            ang *= (1.f - 2.f * rng_next(r0, r1)) * p1.x;
            sincosf(ang, &st, &ct);
            rotate(L.vx, L.vy, L.vz, st, ct, sphi, cphi);
            canfocus = false;
            located = true;
            break;
        }
        case kSrcHyperboloid: {
            float sphi, cphi;
            sincosf(kTWO_PI * rng_next(r0, r1), &sphi, &cphi);
            const float r = sqrtf(0.5f * -logf(rng_next(r0, r1) + kEPS)) * p1.x;
            const float a = __fdividef(-p1.y, p1.z), b = rsqrtf(r * r + p1.z * p1.z);
            // displacement from the source and direction, in the beam's frame (beam along +z)
            float qx = r * (cphi - a * sphi), qy = r * (sphi + a * cphi), qz = 0.f;
            const float dx = -r * sphi * b, dy = r * cphi * b, dz = p1.z * b;
            if (L.vz > -1.f + kEPS && L.vz < 1.f - kEPS) {
                float t = 1.f - L.vz * L.vz;
                const float st = sqrtf(t);
                t = rsqrtf(t);
                const float cp = L.vx * t, sp = L.vy * t, vz = L.vz;
                const float ax = qx * cp * vz - qy * sp, ay = qx * sp * vz + qy * cp, az = -qx * st;
                qx = ax; qy = ay; qz = az;
                L.vx = dx * cp * vz - dy * sp + dz * cp * st;
                L.vy = dx * sp * vz + dy * cp + dz * sp * st;
                L.vz = -dx * st + dz * vz;
            } else {
                L.vx = dx; L.vy = dy; L.vz = (L.vz > 0.f) ? dz : -dz;
            }
            L.px += qx; L.py += qy; L.pz += qz;
            canfocus = false;
            break;
        }
        case kSrcLine: case kSrcSlit: {
            float r = rng_next(r0, r1);
            L.px += r * p1.x; L.py += r * p1.y; L.pz += r * p1.z;
            if (P.srctype == kSrcLine) {
                float sphi, cphi;
                r = rsqrtf(p1.x * p1.x + p1.y * p1.y + p1.z * p1.z);
                const float ax = p1.x * r, ay = p1.y * r, az = p1.z * r;
                if (p2.x > 0.f) {
                    // direction: srcdir made normal to the line, turned about it by up to p2.x
                    r = L.vx * ax + L.vy * ay + L.vz * az;
                    L.vx -= r * ax; L.vy -= r * ay; L.vz -= r * az;
                    r = rsqrtf(L.vx * L.vx + L.vy * L.vy + L.vz * L.vz);
                    L.vx *= r; L.vy *= r; L.vz *= r;
                    sincosf(p2.x * (2.f * rng_next(r0, r1) - 1.f), &sphi, &cphi);
                    const float cx = ay * L.vz - az * L.vy, cy = az * L.vx - ax * L.vz, cz = ax * L.vy - ay * L.vx;
                    L.vx = L.vx * cphi + cx * sphi; L.vy = L.vy * cphi + cy * sphi; L.vz = L.vz * cphi + cz * sphi;
                } else {
                    L.vx = ax; L.vy = ay; L.vz = az;
                    sincosf(kTWO_PI * rng_next(r0, r1), &sphi, &cphi);
                    rotate(L.vx, L.vy, L.vz, 1.f, 0.f, sphi, cphi);
                }
            } else if (p2.x > 0.f || p2.y > 0.f) {
                float sphi, cphi;
                sincosf(kTWO_PI * rng_next(r0, r1), &sphi, &cphi);
                r = sqrtf(2.f * -logf(rng_next(r0, r1) + kEPS));
                cphi *= p2.x * r;
                sphi *= p2.y * r * rsqrtf(p1.x * p1.x + p1.y * p1.y + p1.z * p1.z);
                const float nx = p1.y * L.vz - p1.z * L.vy, ny = p1.z * L.vx - p1.x * L.vz, nz = p1.x * L.vy - p1.y * L.vx;
                cphi *= rsqrtf(nx * nx + ny * ny + nz * nz);
                L.vx += cphi * nx + sphi * p1.x;
                L.vy += cphi * ny + sphi * p1.y;
                L.vz += cphi * nz + sphi * p1.z;
                r = rsqrtf(L.vx * L.vx + L.vy * L.vy + L.vz * L.vz);
                L.vx *= r; L.vy *= r; L.vz *= r;
            }
            ox = sp.x + p1.x * 0.5f; oy = sp.y + p1.y * 0.5f; oz = sp.z + p1.z * 0.5f;
            canfocus = (P.srctype == kSrcSlit);
            break;
        }
        case kSrcPencil:            // only with a launch-angle table (MCX's non-pencil path then)
            break;
        default:
            return false;
        }
        if (fabsf(L.w) <= P.minenergy) continue;
        if (FULL && P.nangle > 0) {
            // launch zenith angle from the user's inverse CDF (src/mcx_core.cu:1581-1605): read
            // directly with a positive focal length, else interpolated; the azimuth is uniform
            const int na = P.nangle;
            const float f = sfocal;
            float ang = rng_next(r0, r1), c;
            if (sfocus == kFocusLength && f > 0.f) {
                ang = fminf(ang * na, na - kEPS);
                c = __ldg(P.angleinvcdf + min((int)ang, na - 1));
            } else {
                ang = fminf(ang * (na - 1), na - 1 - kEPS);
                const float fr = ang - (int)ang;
                c = (1.f - fr) * __ldg(P.angleinvcdf + min((int)ang, na - 1)) +
                    fr * __ldg(P.angleinvcdf + min((int)ang + 1, na - 1));
            }
            float st, ct, sphi, cphi;
            sincosf(c * 3.14159265358979f, &st, &ct);
            sincosf(kTWO_PI * rng_next(r0, r1), &sphi, &cphi);
            // MCX resets the direction to srcdir for focal lengths in [0, 1.5)
            if (sfocus == kFocusNone || (sfocus == kFocusLength && f >= 0.f && f < 1.5f)) {
                L.vx = sv.x; L.vy = sv.y; L.vz = sv.z;
            }
            rotate(L.vx, L.vy, L.vz, st, ct, sphi, cphi);
        } else if (canfocus && sfocus != kFocusNone) {
            // the host classifies the focal length: fast-math code must not test for NaN or inf
            const float f = sfocal;
            float sphi, cphi, st, ct;
            if (sfocus == kFocusIsotropic) {                       // NaN focal length
                sincosf(kTWO_PI * rng_next(r0, r1), &sphi, &cphi);
                sincosf(acosf(2.f * rng_next(r0, r1) - 1.f), &st, &ct);
                rotate(L.vx, L.vy, L.vz, st, ct, sphi, cphi);
            } else if (sfocus == kFocusLambertian) {               // -inf focal length
                sincosf(kTWO_PI * rng_next(r0, r1), &sphi, &cphi);
                st = sqrtf(rng_next(r0, r1));
                ct = sqrtf(1.f - st * st);
                rotate(L.vx, L.vy, L.vz, st, ct, sphi, cphi);
            } else {                                                    // converging / diverging
                const float sg = (f > 0.f) ? 1.f : -1.f;
                ox += f * L.vx; oy += f * L.vy; oz += f * L.vz;
                L.vx = sg * (ox - L.px); L.vy = sg * (oy - L.py); L.vz = sg * (oz - L.pz);
                const float k = rsqrtf(L.vx * L.vx + L.vy * L.vy + L.vz * L.vz);
                L.vx *= k; L.vy *= k; L.vz *= k;
            }
        }
        // launch voxel: the host's for point sources, else where the photon stands
        unsigned lab = 0u;
        if (located && !ALT) {
            L.idx = P.src_idx;
            L.ix = P.src_fx; L.iy = P.src_fy; L.iz = P.src_fz;
            lab = P.src_label;
        } else {
            const int fx = (int)floorf(L.px), fy = (int)floorf(L.py), fz = (int)floorf(L.pz);
            if (L.px >= 0.f && L.py >= 0.f && L.pz >= 0.f && L.px < P.d_fnx && L.py < P.d_fny && L.pz < P.d_fnz &&
                in_grid(P, fx, fy, fz)) {
                L.idx = (unsigned)fz * P.dimxy + (unsigned)fy * (unsigned)P.nx + (unsigned)fx;
                L.ix = fx; L.iy = fy; L.iz = fz;
                lab = voxel_load<WORDS>(P, L.idx);
            }
        }
        if (voxel_med<WORDS>(lab) == 0u) {
            const int id = skip_void<WORDS>(P, L);
            if (id < 0) continue;
            L.idx = (unsigned)id;
            lab = voxel_load<WORDS>(P, L.idx);
        }
        if (voxel_med<WORDS>(lab) == 0u || fabsf(L.w) <= P.minenergy) continue;
        L.label = lab;
        return true;
    }
    return false;
}

// Accumulation into the global field.  FP64 in the reference-accuracy twin; in FP32, a large
// contribution (a spilled or flushed shared-memory tile value) goes through the two-copy
// scheme of src/mcx_core.cu:2246-2253 -- whenever the primary copy holds more than kMaxAccum
// in magnitude, a fixed kMaxAccum moves to the shadow copy, which only ever sums multiples of
// kMaxAccum and so stays exact -- while single deposits are fire-and-forget reductions.
__device__ __forceinline__ void field_add_large(const KParams& P, size_t addr, float v) {
    if (P.field64) {
        atomicAdd(P.field64 + addr, (double)v);
        return;
    }
    const float old = atomicAdd(P.field + addr, v);
    if (fabsf(old) > kMaxAccum) {
        const float m = (old > 0.f) ? kMaxAccum : -kMaxAccum;
        atomicAdd(P.field + addr, -m);
        atomicAdd(P.shadow + addr, m);
    }
}

__device__ __forceinline__ void field_add_small(const KParams& P, size_t addr, float v) {
    if (P.field64) atomicAdd(P.field64 + addr, (double)v);
    else atomicAdd(P.field + addr, v);
}

// Photon sharing (src/mcx_core.cu:2259-2275): one deposit of a unit-weight photon feeds every
// pattern's channel with that pattern's weight at the photon's starting pixel; the channels of
// a voxel and gate are adjacent, (voxel + gate x nvox) x srcnum + pattern.
__device__ __forceinline__ void share_deposit(const KParams& P, unsigned pix, size_t addr, float v) {
    const float* pw = P.srcpattern + (size_t)pix * (unsigned)P.srcnum;
    const size_t base = addr * (unsigned)P.srcnum;
    for (int i = 0; i < P.srcnum; i++) {
        const float f = __ldg(pw + i);
        if (f != 0.f) field_add_small(P, base + i, v * f);
    }
}

// Shared-memory carve-up of one CTA.
// One trajectory record (savedebugdata, src/mcx_core.cu:427-442): photon id as uint bits, the
// position in grid units, the weight and the source id (0: one source).  Records past traj_max
// are counted but not written.
// With istrajstokes (polarised runs) the record continues with the Stokes vector (453-462).
__device__ __forceinline__ void traj_save(const KParams& P, unsigned id, float x, float y, float z, float w, int src,
                                          const float* stk, unsigned stride) {
    const unsigned pos = atomicAdd(P.traj_count, 1u);
    if (pos < P.traj_max) {
        float* r = P.traj + (size_t)pos * (unsigned)P.traj_reclen;
        if (P.traj_reclen == 10) {
            r[6] = stk[0];
            r[7] = stk[stride];
            r[8] = stk[2 * stride];
            r[9] = stk[3 * stride];
        }
        r[0] = __uint_as_float(id);
        r[1] = x;
        r[2] = y;
        r[3] = z;
        r[4] = w;
        r[5] = (float)src;
    }
}

struct Smem {
    float4* prop;                 // medianum x (mua, mus, g, n)
    unsigned long long* pool;     // per warp: next, end of its photon-index pool
    int* drained;                 // per warp: the global photon counter is exhausted
    unsigned* wcount;             // per warp: launches tried, deposits into the tile, photons run
    float* wlaunch;               // per thread: launch weight of its photon
    unsigned* left;               // per thread, MCX stream mode: photons still to run from its stream
    unsigned* step0;              // per thread: the lane's step count when its photon started
    int* nscat0;                  // per thread, detector runs: nscat at the last change of medium
    float* tally;                 // kNumEnergy x blockDim, FP32 per-thread partial sums
    float* ppath;                 // partialdata x blockDim (detector runs)
    unsigned long long* seed0;    // 2 x blockDim, general variant: generator state at launch
    float* rw;                    // per thread, replay: detected weight of the photon
    float* rtof;                  // per thread, replay: its time of flight
    float* rcos;                  // per thread, RF replay: cos and sin of omega x time of flight
    int* rbin;                    // per thread, replay: its field block (gate + detector offset), -1 none
    unsigned* pid;                // per thread, trajectories: the photon's id
    float* stokes;                // 4 x blockDim, polarised light: the photon's Stokes vector (I, Q, U, V)
    unsigned* spix;               // per thread, photon sharing: the pattern pixel of its photon
    int* ssrc;                    // per thread, extra sources: the source (1-based) of its photon
    unsigned* tile;               // deposit tile, fixed point (weight x d_tile_scale)
};

template <bool SAVEDET, bool FULL>
__device__ __forceinline__ Smem carve(const KParams& P, unsigned char* raw) {
    Smem s;
    const unsigned warps = blockDim.x >> 5;
    s.prop = reinterpret_cast<float4*>(raw);
    s.pool = reinterpret_cast<unsigned long long*>(s.prop + P.medianum);
    s.drained = reinterpret_cast<int*>(s.pool + 2 * warps);
    s.wcount = reinterpret_cast<unsigned*>(s.drained + warps);
    s.left = s.wcount + 3 * warps;
    s.step0 = s.left + blockDim.x;
    s.nscat0 = reinterpret_cast<int*>(s.step0 + blockDim.x);
    s.wlaunch = reinterpret_cast<float*>(s.nscat0 + blockDim.x);
    s.tally = s.wlaunch + blockDim.x;
    s.ppath = s.tally + kNumEnergy * blockDim.x;
    float* end = s.ppath + (SAVEDET ? P.partialdata * blockDim.x : 0u);
    if (FULL) {
        // 8-byte aligned: everything before is a multiple of 4 bytes
        s.seed0 = reinterpret_cast<unsigned long long*>((reinterpret_cast<uintptr_t>(end) + 7u) & ~uintptr_t(7));
        s.rw = reinterpret_cast<float*>(s.seed0 + 2 * blockDim.x);
        s.rtof = s.rw + blockDim.x;
        s.rcos = s.rtof + blockDim.x;                 // cos, then sin, blockDim.x each
        s.rbin = reinterpret_cast<int*>(s.rcos + 2 * blockDim.x);
        s.pid = reinterpret_cast<unsigned*>(s.rbin + blockDim.x);
        s.stokes = reinterpret_cast<float*>(s.pid + blockDim.x);
        s.spix = reinterpret_cast<unsigned*>(s.stokes + 4 * blockDim.x);
        s.ssrc = reinterpret_cast<int*>(s.spix + blockDim.x);
        end = reinterpret_cast<float*>(s.ssrc + blockDim.x);
    }
    s.tile = reinterpret_cast<unsigned*>(end);
    return s;
}

// Per-medium partial path (flag P) and scattering count (flag S) of a detector run
// (src/mcx_core.cu:1970-1981, 2152-2165): the reference adds every step's length and every
// scattering event to the slot of the current medium; here they are summed in registers while
// the medium stays the same and added to the slot of medium `m` when it changes.
__device__ __forceinline__ void flush_segment(const KParams& P, const Smem& S, int tid, int B, int m, float& segp,
                                              int nscat) {
    if (m > 0) {
        const unsigned fS = (P.savedetflag >> 1) & 1u, fP = (P.savedetflag >> 2) & 1u;
        if (fS) S.ppath[(unsigned)(m - 1) * B + tid] += (float)(nscat - S.nscat0[tid]);
        if (fP) S.ppath[((unsigned)P.nmedia_det * fS + (unsigned)(m - 1)) * B + tid] += segp;
    }
    S.nscat0[tid] = nscat;
    segp = 0.f;
}

// MINB: CTAs of 256 threads the register budget is sized for (4 -> 64 registers, 3 -> 85, 2 -> 128).
// MODE 0: pencil beam, flux / fluence / energy.  MODE 1: adds per-photon sampling of the other
// source shapes.  MODE 2: adds replay, seed saving and the replay / path-length outputs.
template <bool REFLECT, bool SAVEDET, int MINB, int MODE>
__global__ void __launch_bounds__(256, MINB) transport_kernel(const __grid_constant__ KParams P) {
    constexpr bool AREA = MODE >= 1;
    constexpr bool FULL = MODE >= 2;
    constexpr bool WORDS = MODE >= 3;
    constexpr bool SVMC = MODE == 4;       // split voxels (MEDIA_2LABEL_SPLIT)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Smem S = carve<SAVEDET, FULL>(P, smem_raw);
    const int tid = threadIdx.x;
    const int B = blockDim.x;
    const unsigned lane = tid & 31u;
    const unsigned warp = tid >> 5;

    for (int i = tid; i < P.medianum; i += B) S.prop[i] = P.prop[i];
    for (int k = 0; k < kNumEnergy; k++) S.tally[k * B + tid] = 0.f;
    const int tile_elems = P.tile_on ? P.tnx * P.tny * P.tnz * P.tng : 0;
    for (int i = tid; i < tile_elems; i += B) S.tile[i] = 0u;
    if (lane == 0) {
        S.pool[2 * warp] = 0ull;
        S.pool[2 * warp + 1] = 0ull;
        S.drained[warp] = (P.src_ok == 0);
        S.wcount[3 * warp] = 0u;
        S.wcount[3 * warp + 1] = 0u;
        S.wcount[3 * warp + 2] = 0u;
    }
    __syncthreads();

    // Time runs in grid-length units (sum of len*n): the time bin is one FMA away and the
    // window tests compare against pre-divided bounds.  Launch-uniform constants are read from
    // the parameter block where they are used.
#define inv_c0 P.d_inv_c0
#define tw0 P.d_tw0
#define tw1 P.d_tw1
#define bin_a P.d_bin_a
#define bin_b P.d_bin_b
#define n0 P.d_n0
#define fnx P.d_fnx
#define fny P.d_fny
#define fnz P.d_fnz
#define gscat P.d_gscat
#define tx0 P.d_tx0
#define ty0 P.d_ty0
#define tz0 P.d_tz0
#define tx1 P.d_tx1
#define ty1 P.d_ty1
#define tz1 P.d_tz1

    bool alive = false;
    // photon state
    float px = 0.f, py = 0.f, pz = 0.f, w = 0.f;
    float vx = 0.f, vy = 0.f, vz = 1.f, rvx = 0.f, rvy = 0.f, rvz = 0.f;
    float pscat = 0.f, t = 0.f, pathlen = 0.f, w0 = 0.f;
    float eabs = 0.f;                   // absorbed weight recorded in the field (the rest goes to the
                                        // kEAbsOther tally as it happens)
    float fx = 0.f, fy = 0.f, fz = 0.f; // integer voxel coordinates, as floats
    // detector runs: path length in the current medium since the last change of medium (the
    // scattering count since then is nscat minus its value then, kept in shared memory)
    float segp = 0.f;
    int nscat = -1;
    // det: the current voxel has the detector bit.  carry: the detector bit of the reference's
    // `isdet` as it stands at the end of a step -- the new voxel's (clear outside, where isdet
    // holds a boundary code), which after a reflection still describes the voxel bounced off;
    // it feeds the next step's mediaidold.
    unsigned idx = 0u;
    bool det = false, carry = false;
    int med = 0;
    float4 pr = make_float4(0.f, 0.f, 0.f, 1.f);
    SplitVoxel sv{0, 0, false, false, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool sv_test = false;           // test the plane on the next flight (off right after crossing it)
    unsigned long long r0 = 0ull, r1 = 0ull;
    unsigned c_step = 0u, c_scat = 0u, c_dep = 0u;
    S.left[tid] = 0u;

    while (true) {
        // ---- relaunch lanes that have no photon (warp-uniform control flow) ------------------
        unsigned need = __ballot_sync(kFull, !alive);
        if (need) {
            bool start = false;
            // MCX stream mode: a stream with photons left continues with its RNG state
            if (!alive && P.seed_mode == 1) {
                const unsigned left = S.left[tid];
                if (left > 0u) {
                    S.left[tid] = left - 1u;
                    start = true;
                    if (FULL && P.traj) S.pid[tid] += 1u;       // the stream's next photon
                }
            }
            const unsigned want = __ballot_sync(kFull, !alive && !start);
            if (want && !S.drained[warp]) {
                const unsigned n = __popc(want);
                const unsigned rank = __popc(want & ((1u << lane) - 1u));
                unsigned long long pool_next = S.pool[2 * warp], pool_end = S.pool[2 * warp + 1];
                const unsigned long long avail = pool_end - pool_next;
                unsigned long long mine = pool_next + rank;
                if (avail < n) {
                    // reserve at least what the dead lanes need, normally a whole chunk
                    const unsigned long long take = max((unsigned long long)P.chunk, (unsigned long long)(n - avail));
                    unsigned long long base = 0ull;
                    if (lane == 0) base = atomicAdd(P.work, take);
                    base = __shfl_sync(kFull, base, 0);
                    if (rank >= avail) mine = base + (rank - avail);
                    pool_next = base + (n - avail);
                    pool_end = base + take;
                    if (lane == 0 && base >= P.d_nwork) S.drained[warp] = 1;
                } else {
                    pool_next += n;
                }
                __syncwarp();               // every lane has read the pool before lane 0 rewrites it
                if (lane == 0) {
                    S.pool[2 * warp] = pool_next;
                    S.pool[2 * warp + 1] = pool_end;
                }
                // the pool and the drained flag are read by every lane at the next refill: a warp
                // barrier makes lane 0's writes visible to them (the ballots in between order the
                // lanes but not their shared-memory accesses, and the compiler may keep a lane's
                // earlier reads of these words in registers across them)
                __syncwarp();
                if (!alive && !start && mine < P.d_nwork) {
                    if (FULL && P.replay) {
                        // a detected photon again: its saved launch state and detection record
                        // (src/mcx_core.cu:1203-1211)
                        r0 = __ldg(P.replay_seed + 2 * mine);
                        r1 = __ldg(P.replay_seed + 2 * mine + 1);
                        const float tof = __ldg(P.replay_tof + mine);
                        int bin = (int)floorf((tof - P.twin0) * P.Rtstep);
                        if (bin < 0 || bin >= P.maxgate) {
                            bin = -1;           // detected outside this gate group: nothing to add
                        } else if (P.replaydet == -1) {
                            bin += ((__ldg(P.replay_detid + mine) & 0xFFFF) - 1) * P.maxgate;
                        }
                        S.rw[tid] = __ldg(P.replay_w + mine);
                        S.rtof[tid] = tof;
                        S.rbin[tid] = bin;
                        if (P.outputtype == kOutRF || P.outputtype == kOutRFmus) {
                            // modulation phase of the detected photon (src/mcx_core.cu:1700-1703)
                            float sn, cs;
                            sincosf(P.omega * tof, &sn, &cs);
                            S.rcos[tid] = cs;
                            S.rcos[B + tid] = sn;
                        }
                        start = true;
                    } else if (P.seed_mode == 1) {
                        // MCX's per-thread stream `mine`: four host seed words
                        // (src/mcx_rand_xorshift128p.cu:79-82), then its share of photons in sequence
                        const unsigned cnt = P.mcx_per + ((unsigned)mine < P.mcx_odd ? 1u : 0u);
                        if (cnt) {
                            const uint4 sw = __ldg(reinterpret_cast<const uint4*>(P.mcx_words) + mine);
                            r0 = ((unsigned long long)sw.x << 32) | sw.y;
                            r1 = ((unsigned long long)sw.z << 32) | sw.w;
                            S.left[tid] = cnt - 1u;
                            start = true;
                            // MCX's id: the thread's first photon index plus its 1-based count
                            if (FULL && P.traj)
                                S.pid[tid] = (unsigned)mine * P.mcx_per + min((unsigned)mine, P.mcx_odd) + 1u;
                        }
                    } else {
                        seed_photon(P.seed, P.photon_offset + mine, r0, r1);
                        start = true;
                    }
                    if (FULL && P.traj && (P.seed_mode != 1 || P.replay)) S.pid[tid] = (unsigned)(P.photon_offset + mine) + 1u;
                }
            }
            if (FULL && start && P.saveseed) {      // state at launch (src/mcx_core.cu:1213-1215)
                S.seed0[2 * tid] = r0;
                S.seed0[2 * tid + 1] = r1;
            }
            // extra sources (src/mcx_core.cu:1217-1227): the photon's source, drawn after the seed
            // is saved when every source runs (srcid 0 or -1)
            const float4* alt = nullptr;
            if (FULL && start && P.nextra) {
                int k = 1;
                if (P.srcid > 1) k = P.srcid;
                else if (P.srcid <= 0) k = (int)(rng_next(r0, r1) * 0.9998f * (P.nextra + 1)) + 1;
                S.ssrc[tid] = k;
                if (k > 1) alt = P.extrasrc + 5 * (k - 2);
            }
            // a replay of one chosen source skips the draw by which the recorded run picked its
            // source among all of them (src/mcx_core.cu:1229-1231)
            if (FULL && start && P.replay && P.srcid >= 1) (void)rng_next(r0, r1);
            bool entered = false;
            if (start && P.srctype == kSrcPencil && !(FULL && (P.nangle > 0 || P.nextra))) {
                // launch (pencil branch of src/mcx_core.cu:1236-1243, 1646-1717; the void
                // skipping and specular loss of skipvoid() are folded into src_* by the host)
                px = P.src_p.x; py = P.src_p.y; pz = P.src_p.z; w = P.src_p.w;
                vx = P.src_v.x; vy = P.src_v.y; vz = P.src_v.z;
                t = P.src_t * inv_c0;
                idx = P.src_idx;
                const unsigned lab = voxel_pick<WORDS>(P, P.src_label, r0, r1);
                med = (int)voxel_med<WORDS>(lab);
                det = voxel_det<WORDS>(lab);
                fx = (float)P.src_fx; fy = (float)P.src_fy; fz = (float)P.src_fz;
                entered = true;
            } else if (AREA && start) {
                Launch L;
                entered = launch_source<WORDS, FULL>(P, r0, r1, L, alt);
                if (entered) {
                    px = L.px; py = L.py; pz = L.pz; w = L.w;
                    vx = L.vx; vy = L.vy; vz = L.vz;
                    t = L.t;
                    idx = L.idx;
                    const unsigned lab = voxel_pick<WORDS>(P, L.label, r0, r1);
                    med = (int)voxel_med<WORDS>(lab);
                    det = voxel_det<WORDS>(lab);
                    fx = (float)L.ix; fy = (float)L.iy; fz = (float)L.iz;
                    if (FULL && P.srcnum > 1) S.spix[tid] = L.pix;
                }
            }
            if (entered) {
                rvx = __fdividef(1.f, vx); rvy = __fdividef(1.f, vy); rvz = __fdividef(1.f, vz);
                carry = det;
                S.wlaunch[tid] = w;
                pscat = 0.f; pathlen = 0.f; nscat = -1;
                segp = 0.f;
                if (SAVEDET) S.nscat0[tid] = 0;
                w0 = w; eabs = 0.f;
                S.step0[tid] = c_step;
                pr = props_of<WORDS>(P, S.prop, (unsigned)med, idx);
                if constexpr (SVMC) {           // src/mcx_core.cu:1246-1251, 1679
                    split_voxel_at(P, idx, fx, fy, fz, px, py, pz, sv);
                    pr = S.prop[sv.tissue()];
                    sv_test = true;
                }
                if (SAVEDET)
                    for (unsigned k = 0; k < P.partialdata; k++) S.ppath[k * B + tid] = 0.f;
                if (FULL && P.polarized) {      // src/mcx_core.cu:1254-1256
                    S.stokes[tid] = P.srciquv.x;
                    S.stokes[B + tid] = P.srciquv.y;
                    S.stokes[2 * B + tid] = P.srciquv.z;
                    S.stokes[3 * B + tid] = P.srciquv.w;
                }
                if (FULL && P.traj) traj_save(P, S.pid[tid], px, py, pz, w, (P.nextra && P.srcid <= 0) ? S.ssrc[tid] : 0, S.stokes + tid, B);     // 1681-1687
                alive = true;
            }
            const unsigned attempted = __ballot_sync(kFull, start), ran = __ballot_sync(kFull, entered);
            if (lane == 0) {
                S.wcount[3 * warp] += __popc(attempted);
                S.wcount[3 * warp + 2] += __popc(ran);
            }
            need = __ballot_sync(kFull, !alive);
            if (need == kFull && attempted == 0u) break;   // no photon left for any lane of this warp
        }
        if (!alive) continue;

        // ---- one step (src/mcx_core.cu:1888-2514) --------------------------------------------
        c_step++;
        unsigned detflag = 0u;
        bool kill = false;

        if (pscat <= 0.f) {
            // random numbers of this scattering event: MCX's order (scattering length, azimuth,
            // zenith), one generator step each in MCX seeding mode, one step for all three with
            // per-photon streams
            float u_len, u_phi, u_th;
            if (P.seed_mode == 1) {
                u_len = rng_next(r0, r1);
            } else {
                rng_next3(r0, r1, u_len, u_phi, u_th);
            }
            pscat = -__logf(u_len + kEPS);                               // src/mcx_rand_xorshift128p.cu:122
            if (nscat >= 0) {                                           // not the launch flight
                if (P.seed_mode == 1 && !(FULL && P.polarized)) {   // polarised: the rejection loop draws
                    u_phi = rng_next(r0, r1);
                    u_th = rng_next(r0, r1);
                }
                float sphi, cphi;
                __sincosf(kTWO_PI * u_phi, &sphi, &cphi);               // src/mcx_core.cu:1930-1933
                const float g = (nscat > gscat) ? 0.f : pr.z;
                float ct;
                float pol_theta = 0.f, pol_phi = 0.f;
                const float4* mrow = nullptr;
                if (FULL && P.polarized) {
                    // polarised: (theta, phi) from the medium's Mueller table by rejection against
                    // the forward intensity for the photon's Stokes vector (src/mcx_core.cu:1909-1930)
                    mrow = P.smatrix + (size_t)kNAngles * (unsigned)(med - 1);
                    const float si = S.stokes[tid], sq = S.stokes[B + tid], su = S.stokes[2 * B + tid];
                    const float4 m0 = __ldg(mrow);
                    for (int tries = 0; tries < 100000; tries++) {
                        pol_theta = acosf(2.f * rng_next(r0, r1) - 1.f);
                        pol_phi = kTWO_PI * rng_next(r0, r1);
                        float s2p, c2p;
                        sincosf(2.f * pol_phi, &s2p, &c2p);
                        const float lin = sq * c2p + su * s2p;
                        const float4 mt = __ldg(mrow + (int)floorf(pol_theta * kNAngles * (kR_PI - kEPS)));
                        if (rng_next(r0, r1) * (m0.x * si + m0.y * lin) < mt.x * si + mt.y * lin) break;
                    }
                    sincosf(pol_phi, &sphi, &cphi);
                    ct = cosf(pol_theta);
                } else if (FULL && P.nphase > 2) {
                    // user phase function (src/mcx_core.cu:1937-1944): cos(theta) interpolated in
                    // the inverse CDF, whose ends are -1 and 1
                    const int np = P.nphase;
                    const float a = u_th * (np - 1);
                    const float fr = a - (int)a;
                    ct = (1.f - fr) * __ldg(P.invcdf + min((int)a, np - 1)) + fr * __ldg(P.invcdf + min((int)a + 1, np - 1));
                } else if (fabsf(g) > kEPS) {                           // Henyey-Greenstein, 1946-1959
                    const float g2 = g * g;
                    float tmp = __fdividef(1.f - g2, 1.f - g + 2.f * g * u_th);
                    tmp *= tmp;
                    ct = __fdividef(1.f + g2 - tmp, 2.f * g);
                    ct = fmaxf(-1.f, fminf(1.f, ct));
                } else {
                    ct = 2.f * u_th - 1.f;                              // isotropic, 1961-1963
                }
                const float st = (FULL && P.polarized) ? sinf(pol_theta) : sqrtf(fmaxf(0.f, 1.f - ct * ct));
                const float ox0 = vx, oy0 = vy, oz0 = vz;               // direction before the event
                if (SAVEDET && !WORDS && med > 0 && ((P.savedetflag >> 3) & 1u)) {   // momentum transfer, 1970-1993
                    const unsigned fS = (P.savedetflag >> 1) & 1u, fP = (P.savedetflag >> 2) & 1u;
                    S.ppath[((unsigned)P.nmedia_det * (fS + fP) + (unsigned)(med - 1)) * B + tid] += 1.f - ct;
                }
                if (FULL && P.replay && (P.outputtype == kOutWP || P.outputtype == kOutDCS ||
                                         P.outputtype == kOutWPTOF || P.outputtype == kOutRFmus)) {
                    // replay outputs at scattering events (src/mcx_core.cu:2018-2066): detected weight
                    // x (1, momentum transfer 1 - cos, time of flight, or cos / sin of the RF phase)
                    // in the current voxel
                    const int rb = S.rbin[tid];
                    if (rb >= 0) {
                        float q = S.rw[tid];
                        // every source apart: the source's block of (detector) blocks, as at deposits
                        const int sb = (P.nextra && P.srcid < 0)
                                           ? (S.ssrc[tid] - 1) * ((P.replaydet == -1) ? P.detnum : 1) * P.maxgate
                                           : 0;
                        const size_t at = (size_t)idx + (size_t)(rb + sb) * P.nvox;
                        if (P.outputtype == kOutDCS) q *= 1.f - ct;
                        else if (P.outputtype == kOutWPTOF) q *= S.rtof[tid];
                        if (P.outputtype == kOutRFmus) {
                            field_add_small(P, at + P.rf_offset, q * S.rcos[B + tid]);
                            q *= S.rcos[tid];
                        }
                        field_add_small(P, at, q);
                    }
                }
                rotate(vx, vy, vz, st, ct, sphi, cphi);
                if (FULL && P.polarized) {
                    // updatestokes (src/mcx_core.cu:318-352): into the scattering plane, through the
                    // Mueller matrix at theta, back to the new meridian plane, normalised to I = 1
                    float si = S.stokes[tid], sq = S.stokes[B + tid], su = S.stokes[2 * B + tid], sv = S.stokes[3 * B + tid];
                    float s2p, c2p;
                    sincosf(2.f * pol_phi, &s2p, &c2p);
                    const float q1 = sq * c2p + su * s2p, u1 = -sq * s2p + su * c2p;
                    const float4 mt = __ldg(mrow + (int)floorf(pol_theta * kNAngles * (kR_PI - kEPS)));
                    const float I = mt.x * si + mt.y * q1, Q = mt.y * si + mt.x * q1;
                    const float U = mt.z * u1 + mt.w * sv, V = -mt.w * u1 + mt.z * sv;
                    const float den = (vz > -1.f && vz < 1.f) ? (1.f - ct * ct) * (1.f - vz * vz) : 0.f;
                    float ci = 0.f;
                    if (den > 0.f) {
                        ci = ((pol_phi > kPI && pol_phi < kTWO_PI) ? 1.f : -1.f) * (vz * ct - oz0) * rsqrtf(den);
                        ci = fmaxf(-1.f, fminf(ci, 1.f));
                    }
                    const float sn = sqrtf(1.f - ci * ci), c22 = 2.f * ci * ci - 1.f, s22 = 2.f * sn * ci;
                    const float inv = __fdividef(1.f, I);
                    S.stokes[tid] = 1.f;
                    S.stokes[B + tid] = (Q * c22 - U * s22) * inv;
                    S.stokes[2 * B + tid] = (Q * s22 + U * c22) * inv;
                    S.stokes[3 * B + tid] = V * inv;
                    (void)ox0; (void)oy0;
                }
                nscat++;
                rvx = __fdividef(1.f, vx); rvy = __fdividef(1.f, vy); rvz = __fdividef(1.f, vz);
                c_scat++;
                if (FULL && P.traj) traj_save(P, S.pid[tid], px, py, pz, w, (P.nextra && P.srcid <= 0) ? S.ssrc[tid] : 0, S.stokes + tid, B);     // 2068-2074
            } else {
                nscat = 0;
            }
        }

        const float n1 = pr.w;
        if constexpr (SVMC) pr = S.prop[med ? sv.tissue() : 0];
        else pr = props_of<WORDS>(P, S.prop, (unsigned)med, idx);

        // distance to the nearest voxel face (hitgrid, src/mcx_core.cu:493-507)
        const float hx = fabsf((fx + (vx > 0.f ? 1.f : 0.f) - px) * rvx);
        const float hy = fabsf((fy + (vy > 0.f ? 1.f : 0.f) - py) * rvy);
        const float hz = fabsf((fz + (vz > 0.f ? 1.f : 0.f) - pz) * rvz);
        const float dist = fminf(fminf(hx, hy), hz);
        const int axis = (dist == hx) ? 0 : ((dist == hy) ? 1 : 2);

        // src/mcx_core.cu:2101-2109
        const float musp = (nscat >= gscat) ? pr.y * (1.f - pr.z) : pr.y;
        const float sdist = dist * musp;
        const bool stay = !(sdist < pscat);                 // flight ends inside this voxel
        float slen = stay ? pscat : sdist;
        float len = stay ? __fdividef(pscat, musp) : dist;
        bool hit = false;                                   // split voxel: the flight stops on its plane
        if constexpr (SVMC) {
            // ray_plane_intersect (src/mcx_core.cu:747-772) in MCX's arithmetic, so that the same
            // photons take the same decisions: the flight length as the loop recomputes it from
            // the scattering length (2109), the signed distances of both ends, len x d0 / (d0 - d1)
            const float vn = vx * sv.nx + vy * sv.ny + vz * sv.nz;
            if (sv.split && sv_test && vn > 0.f) {
                const float lm = (pr.y == 0.f) ? len : slen / musp;
                const float qx = fmaf(lm, vx, px), qy = fmaf(lm, vy, py), qz = fmaf(lm, vz, pz);
                const float d0 = (px - sv.rx) * sv.nx + (py - sv.ry) * sv.ny + (pz - sv.rz) * sv.nz;
                const float d1 = (qx - sv.rx) * sv.nx + (qy - sv.ry) * sv.ny + (qz - sv.rz) * sv.nz;
                if (!(d0 * d1 > 0.f)) {
                    const float l0 = lm * d0 / (d0 - d1);
                    len = (l0 > 0.f) ? l0 : lm;
                    slen = len * pr.y * ((nscat >= gscat) ? (1.f - pr.z) : 1.f);
                    hit = true;
                }
            }
        }

        px = fmaf(len, vx, px);
        py = fmaf(len, vy, py);
        pz = fmaf(len, vz, pz);
        w *= __expf(-pr.x * len);                                       // 2140
        pscat -= slen;
        t = fmaf(len, pr.w, t);                                         // t += len*n/c0, in grid units
        pathlen += len;
        // step cap, checked every 1024 steps of the lane against its step count at launch
        if ((c_step & 1023u) == 0u && c_step - S.step0[tid] >= P.step_cap) {
            atomicOr(P.errflag, kErrStepCap);
            kill = true;
        }

        const unsigned detold = carry ? kDET_MASK : 0u;   // mediaidold's detector bit (src/mcx_core.cu:2167)
        const int medold = med;
        bool inside = true;
        int bcf = BC_UNKNOWN;
        const unsigned idxold = idx;
        const float ox = fx, oy = fy, oz = fz;

        if (stay && !hit) {
            carry = det;
        } else if (hit) {
            carry = det;                    // same voxel: the segment up to the plane is deposited below
        }
        if (!stay || hit) {
          if (!hit) {
            // cross the face: only the crossed axis can leave the volume (2169-2186)
            float c, lim, sg;
            unsigned stride;
            if (axis == 0) { sg = (vx > 0.f) ? 1.f : -1.f; fx += sg; c = fx; lim = fnx; stride = 1u; }
            else if (axis == 1) { sg = (vy > 0.f) ? 1.f : -1.f; fy += sg; c = fy; lim = fny; stride = (unsigned)P.nx; }
            else { sg = (vz > 0.f) ? 1.f : -1.f; fz += sg; c = fz; lim = fnz; stride = P.dimxy; }
            inside = (c >= 0.f) && (c < lim);
            if (inside) {
                idx = (sg > 0.f) ? idx + stride : idx - stride;
                if (idx >= P.nvox) {
                    // the voxel index has lost step with the coordinates: never read or write out
                    // of the volume; the photon leaves and the host reports the error
                    atomicOr(P.errflag, kErrIndex);
                    inside = false;
                }
            }
            if (inside) {
                const unsigned lab = voxel_pick<WORDS>(P, voxel_load<WORDS>(P, idx), r0, r1);
                med = (int)voxel_med<WORDS>(lab);
                det = voxel_det<WORDS>(lab);
            } else {
                med = 0;
                idx = (c < 0.f) ? kOUT_MIN : kOUT_MAX;
                bcf = P.bc[(idx == kOUT_MAX) * 3 + axis];
                det = false;                // a boundary code, never the detector bit
            }
            carry = det;
          }

            // deposit into the voxel just left (or the split voxel's tissue just left), time bin
            // taken at exit (2191-2292)
            bool rec = false;
            if (P.save2pt && t >= tw0 && t < tw1) {
                // the window test above runs on t in grid units, the bin on t x bin_a - bin_b: at a
                // window that does not start at 0 the two roundings can disagree by one ulp, so a
                // deposit that passed the test may compute bin -1; it belongs to the first gate (MCX's
                // (t - twin0) x Rtstep is exactly >= 0 there), and must never index below the field
                int tshift = (P.maxgate > 1) ? min(P.maxgate - 1, max(0, (int)floorf(fmaf(t, bin_a, -bin_b)))) : 0;
                float weight;
                if (P.outputtype == kOutEnergy) {
                    weight = w0 - w;
                } else if (!FULL || P.outputtype <= kOutFluence) {
                    weight = (pr.x < kEPS) ? (w0 * pathlen) : __fdividef(w0 - w, pr.x);
                } else if (P.outputtype == kOutL) {
                    weight = w0 * pathlen;                  // total path length per voxel
                } else if (P.replay && (P.outputtype == kOutJacobian || P.outputtype == kOutWLTOF)) {
                    // mua Jacobian: detected weight x path in the voxel (x time of flight)
                    const int rb = S.rbin[tid];
                    weight = (rb < 0) ? 0.f : S.rw[tid] * pathlen * (P.outputtype == kOutWLTOF ? S.rtof[tid] : 1.f);
                    tshift = rb;
                } else if (P.replay && P.outputtype == kOutRF) {
                    // RF mua Jacobian (src/mcx_core.cu:2207-2256): -(detected weight x path) x
                    // cos(omega t) here, x sin(omega t) in the imaginary half
                    const int rb = S.rbin[tid];
                    weight = (rb < 0) ? 0.f : -S.rw[tid] * pathlen * S.rcos[tid];
                    if (rb >= 0) {
                        const int sb = (P.nextra && P.srcid < 0)
                                           ? (S.ssrc[tid] - 1) * ((P.replaydet == -1) ? P.detnum : 1) * P.maxgate
                                           : 0;
                        field_add_small(P, (size_t)idxold + (size_t)(rb + sb) * P.nvox + P.rf_offset,
                                        -S.rw[tid] * pathlen * S.rcos[B + tid]);
                    }
                    tshift = rb;
                } else {
                    weight = 0.f;                           // scattering-event outputs (below)
                }
                if (weight != 0.f) {
                    rec = true;
                    c_dep++;
                    // all sources kept apart (srcid -1): one block of gates per source (2225-2227)
                    // (in an all-detector replay a source's block holds one block per detector)
                    const int sblk = (FULL && P.nextra && P.srcid < 0)
                                         ? (S.ssrc[tid] - 1) * ((P.replay && P.replaydet == -1) ? P.detnum : 1) * P.maxgate
                                         : 0;
                    const size_t addr = (size_t)idxold + (size_t)(tshift + sblk) * P.nvox;
                    // the index range of the tile box (empty without a tile) screens most deposits out
                    // with one compare before the box test
                    if (FULL && P.srcnum > 1) {
                        share_deposit(P, S.spix[tid], addr, weight);
                    } else if (idxold - P.d_tile_lo < P.d_tile_span && weight > 0.f && ox >= tx0 && ox < tx1 && oy >= ty0 &&
                        oy < ty1 && oz >= tz0 && oz < tz1 && (unsigned)(tshift - P.tg0) < (unsigned)P.tng) {
                        const int ti = (((tshift - P.tg0) * P.tnz + (int)(oz - tz0)) * P.tny + (int)(oy - ty0)) * P.tnx +
                                       (int)(ox - tx0);
                        // exact fixed-point sum: millions of equal first-flight deposits near the
                        // source carry no rounding bias.  0 <= weight * scale < 2^23, so adding 2^23
                        // leaves its rounded integer value in the low mantissa bits (FP32 pipes only).
                        // The add whose result crosses kTileFlushUnits moves that many units to the
                        // global field; the slot never exceeds 2^31 + 256 * 2^23 < 2^32.
                        const unsigned q = __float_as_uint(fmaf(weight, P.d_tile_scale, 8388608.f)) - 0x4B000000u;
                        const unsigned old = atomicAdd(S.tile + ti, q);
                        if (old < kTileFlushUnits && old + q >= kTileFlushUnits) {
                            atomicSub(S.tile + ti, kTileFlushUnits);
                            field_add_large(P, addr, P.d_tile_flush);
                        }
                        atomicAdd(S.wcount + 3 * warp + 1, 1u);
                    } else {
                        field_add_small(P, addr, weight);
                    }
                }
            }
            if (rec) eabs += w0 - w;
            else S.tally[kEAbsOther * B + tid] += w0 - w;
            w0 = w;
            segp += pathlen;
            pathlen = 0.f;

            if constexpr (SVMC) {
                // a new voxel: its tissue at the photon's position; the plane: the other tissue
                // (src/mcx_core.cu:2295-2303)
                if (!hit) {
                    if (inside && med) split_voxel_at(P, idx, fx, fy, fz, px, py, pz, sv);
                    sv_test = true;
                } else {
                    sv.nx = -sv.nx; sv.ny = -sv.ny; sv.nz = -sv.nz;
                    sv.isup = !sv.isup;
                    sv_test = false;
                }
            }

            // leaving into a 0 voxel or the outside without reflection (2307-2354)
            if (med == 0 && ((!REFLECT || n1 == n0) || (bcf == BC_UNKNOWN && !P.doreflect) || bcf == BC_ABSORB ||
                             bcf == BC_CYCLIC) && bcf != BC_MIRROR)
                kill = true;
            // entering a split voxel's tissue 0 (its background) without reflection
            if (SVMC && inside && med && !sv.isup && sv.lo == 0 && (!REFLECT || n1 == n0)) kill = true;
        }
        if (t > tw1) kill = true;

        if (kill && !inside && bcf == BC_CYCLIC) {                      // 2311-2335
            const float span = (axis == 0) ? fnx : ((axis == 1) ? fny : fnz);
            const float shift = (idx == kOUT_MIN) ? span : -span;
            if (axis == 0) { px = nextafter_mcx(roundf(px + shift), (vx > 0.f) - (vx < 0.f), P.maxvoidstep); fx = floorf(px); }
            else if (axis == 1) { py = nextafter_mcx(roundf(py + shift), (vy > 0.f) - (vy < 0.f), P.maxvoidstep); fy = floorf(py); }
            else { pz = nextafter_mcx(roundf(pz + shift), (vz > 0.f) - (vz < 0.f), P.maxvoidstep); fz = floorf(pz); }
            if (fx >= 0.f && fx < fnx && fy >= 0.f && fy < fny && fz >= 0.f && fz < fnz) {
                idx = (unsigned)fz * P.dimxy + (unsigned)fy * (unsigned)P.nx + (unsigned)fx;
                const unsigned lab = voxel_pick<WORDS>(P, voxel_load<WORDS>(P, idx), r0, r1);
                med = (int)voxel_med<WORDS>(lab);
                det = voxel_det<WORDS>(lab);
                carry = det;
                if constexpr (SVMC) {
                    if (med) split_voxel_at(P, idx, fx, fy, fz, px, py, pz, sv);
                    sv_test = true;
                }
                if (SAVEDET && !WORDS && med != medold) flush_segment(P, S, tid, B, medold, segp, nscat);
                continue;
            }
        }
        if (kill) {
            detflag = (!inside && P.bc[((idx == kOUT_MAX) ? 9 : 6) + axis]) ? kOUT_MIN : (detold & kDET_MASK);
        } else {
            // Russian roulette (2357-2378); off when minenergy is 0
            if (P.minenergy > 0.f && fabsf(w) < P.minenergy) {
                if (rng_next(r0, r1) * 10.f <= 1.f) {
                    w *= 10.f;
                } else {
                    kill = true;
                    detflag = detold & kDET_MASK;
                }
            }
            // Fresnel reflection / refraction at the split voxel's plane (reflectray,
            // src/mcx_core.cu:784-830, 2386-2404): the normal turned back to point along the flight
            if (SVMC && REFLECT && !kill && hit) {
                const float nlo = S.prop[sv.lo].w, nup = S.prop[sv.up].w;
                if (nlo != nup) {
                    sv.nx = -sv.nx; sv.ny = -sv.ny; sv.nz = -sv.nz;
                    const float n2 = S.prop[sv.tissue()].w;           // the tissue entered
                    // (in reflectray's arithmetic: the second term uses the square of the root)
                    const float ic = fabsf(vx * sv.nx + vy * sv.ny + vz * sv.nz);
                    const float a2 = n1 * n1, b2 = n2 * n2;
                    const float c2 = 1.f - a2 / b2 * (1.f - ic * ic);
                    bool refl = true;
                    float ct = 0.f;
                    if (c2 > 0.f) {
                        float re = a2 * ic * ic + b2 * c2;
                        ct = sqrtf(c2);
                        const float im = 2.f * n1 * n2 * ic * ct;
                        float R = (re - im) / (re + im);
                        re = b2 * ic * ic + a2 * ct * ct;
                        R = (R + (re - im) / (re + im)) * 0.5f;
                        refl = rng_next(r0, r1) <= R;
                    }
                    if (refl) {                     // back into the tissue it came from
                        vx -= 2.f * ic * sv.nx; vy -= 2.f * ic * sv.ny; vz -= 2.f * ic * sv.nz;
                        sv.isup = !sv.isup;
                    } else {                        // refracted into the other tissue
                        const float q = n1 / n2;
                        vx = ct * sv.nx + q * (vx - ic * sv.nx);
                        vy = ct * sv.ny + q * (vy - ic * sv.ny);
                        vz = ct * sv.nz + q * (vz - ic * sv.nz);
                        sv.nx = -sv.nx; sv.ny = -sv.ny; sv.nz = -sv.nz;
                        if (sv.tissue() == 0) {     // out into the background: the photon leaves
                            kill = true;
                            detflag = detold & kDET_MASK;
                        }
                    }
                    const float vi = rsqrtf(vx * vx + vy * vy + vz * vz);
                    vx *= vi; vy *= vi; vz *= vi;
                    rvx = __fdividef(1.f, vx); rvy = __fdividef(1.f, vy); rvz = __fdividef(1.f, vz);
                }
                pr = S.prop[sv.tissue()];
            }
            // Fresnel reflection / refraction on crossing (2381-2503)
            if (REFLECT && !kill && !stay && !hit) {
                const float4 prn = SVMC ? S.prop[med ? sv.tissue() : 0] : props_of<WORDS>(P, S.prop, (unsigned)med, idx);
                pr = prn;
                if (((med && P.doreflect) ||
                     (med == 0 && ((bcf == BC_UNKNOWN && P.doreflect) || bcf == BC_REFLECT || bcf == BC_MIRROR))) &&
                    (bcf == BC_MIRROR || n1 != prn.w)) {
                    if (FULL && P.traj) traj_save(P, S.pid[tid], px, py, pz, w, (P.nextra && P.srcid <= 0) ? S.ssrc[tid] : 0, S.stokes + tid, B);     // 2435-2441
                    float Rtotal = 1.f;
                    const float a2 = n1 * n1, b2 = prn.w * prn.w;
                    const float va = (axis == 0) ? vx : ((axis == 1) ? vy : vz);
                    const float cphi = fabsf(va);
                    const float sphi = 1.f - cphi * cphi;
                    const float c2 = 1.f - __fdividef(a2, b2) * sphi;
                    if (c2 > 0.f && bcf != BC_MIRROR) {
                        float ctheta = a2 * cphi * cphi + b2 * c2;
                        const float stheta = 2.f * n1 * prn.w * cphi * sqrtf(c2);
                        Rtotal = __fdividef(ctheta - stheta, ctheta + stheta);
                        ctheta = b2 * cphi * cphi + a2 * c2;
                        Rtotal = (Rtotal + __fdividef(ctheta - stheta, ctheta + stheta)) * 0.5f;
                    }
                    if (Rtotal < 1.f && !(med == 0 && bcf == BC_MIRROR) && rng_next(r0, r1) > Rtotal) {
                        transmit(vx, vy, vz, n1, prn.w, axis);
                        if (med == 0) {
                            kill = true;
                            detflag = (!inside && P.bc[((idx == kOUT_MAX) ? 9 : 6) + axis]) ? kOUT_MIN : (detold & kDET_MASK);
                        } else {
                            rvx = __fdividef(1.f, vx); rvy = __fdividef(1.f, vy); rvz = __fdividef(1.f, vz);
                        }
                    } else {
                        // mirror the direction and nudge the position back into the voxel left
                        if (axis == 0) {
                            vx = -vx;
                            px = nextafter_mcx(rintf(px), (vx > 0.f) - (vx < 0.f), P.maxvoidstep);
                            fx = floorf(px);
                        } else if (axis == 1) {
                            vy = -vy;
                            py = nextafter_mcx(rintf(py), (vy > 0.f) - (vy < 0.f), P.maxvoidstep);
                            fy = floorf(py);
                        } else {
                            vz = -vz;
                            pz = nextafter_mcx(rintf(pz), (vz > 0.f) - (vz < 0.f), P.maxvoidstep);
                            fz = floorf(pz);
                        }
                        rvx = __fdividef(1.f, vx); rvy = __fdividef(1.f, vy); rvz = __fdividef(1.f, vz);
                        idx = idxold;
                        const unsigned lab = voxel_pick<WORDS>(P, voxel_load<WORDS>(P, idx), r0, r1);
                        med = (int)voxel_med<WORDS>(lab);
                        det = voxel_det<WORDS>(lab);     // carry keeps the bounced-off value
                        pr = props_of<WORDS>(P, S.prop, (unsigned)med, idx);
                        if constexpr (SVMC) {
                            // the voxel left, at the reflection point; its background ends the
                            // photon (src/mcx_core.cu:2478-2497)
                            split_voxel_at(P, idx, fx, fy, fz, px, py, pz, sv);
                            pr = S.prop[sv.tissue()];
                            sv_test = true;
                            if (sv.tissue() == 0) {
                                kill = true;
                                detflag = detold & kDET_MASK;
                            }
                        }
                    }
                } else {
                    pr = SVMC ? S.prop[med ? sv.tissue() : 0] : props_of<WORDS>(P, S.prop, (unsigned)medold, idxold);
                }
            }
        }

        if (SAVEDET && !WORDS && (kill || med != medold)) {
            segp += pathlen;        // the last voxel's path when the photon ends inside it, else 0
            flush_segment(P, S, tid, B, medold, segp, nscat);
        }
        if (kill) {
            // terminate: detection and energy bookkeeping (src/mcx_core.cu:1113-1182, 365-417)
            if (FULL && P.traj) traj_save(P, S.pid[tid], px, py, pz, w, (P.nextra && P.srcid <= 0) ? S.ssrc[tid] : 0, S.stokes + tid, B);         // 1116-1122
            if (FULL && P.saveref == 1 && med == 0 && idx != kOUT_MIN && idx != kOUT_MAX && w > 0.f) {
                // diffuse reflectance (1124-1165): the weight leaving into a void voxel of the grid,
                // negated, in that voxel at the photon's gate (a photon before the first gate, which
                // MCX would write below the field, is left out)
                int ts = min(P.maxgate - 1, (int)floorf(fmaf(t, bin_a, -bin_b)));
                if (ts >= 0 && P.nextra && P.srcid < 0) ts += (S.ssrc[tid] - 1) * P.maxgate;
                if (ts >= 0) {
                    if (P.srcnum > 1) share_deposit(P, S.spix[tid], (size_t)idx + (size_t)ts * P.nvox, -w);
                    else field_add_large(P, (size_t)idx + (size_t)ts * P.nvox, -w);
                }
            }
            if (SAVEDET && FULL && P.saveref > 1 && med == 0 && idx != kOUT_MIN && idx != kOUT_MAX && w > 0.f &&
                idx < P.maxdet) {
                // saveexitppath (src/mcx_core.cu:272-285): the exit weight and the weighted partial
                // paths summed into the voxel's record, in MCX's slots (the path of medium 1 shares
                // slot 0 with the weight; the last slot stays empty)
                float* r = P.detp + (size_t)idx * P.reclen;
                atomicAdd(r, w);
                for (int i = 0; i < P.nmedia_det; i++) atomicAdd(r + i, S.ppath[i * B + tid] * w);
            }
            bool detected = false;
            if (SAVEDET && (detflag & kDET_MASK) && (med == 0 || (SVMC && sv.tissue() == 0)) && P.saveref < 2) {
                const int detid = (detflag == kOUT_MIN) ? -1 : find_detector(P, px, py, pz);
                if (detid) {
                    detected = true;
                    const unsigned slot = atomicAdd(P.detcount, 1u);
                    if (FULL && P.saveseed && slot < P.maxdet) {    // src/mcx_core.cu:375-377
                        P.seeddata[2 * slot] = S.seed0[2 * tid];
                        P.seeddata[2 * slot + 1] = S.seed0[2 * tid + 1];
                    }
                    if (slot < P.maxdet) {
                        float* rec = P.detp + (size_t)slot * P.reclen;
                        unsigned k = 0;
                        // with every source running, the source id sits above bit 16 (381-384)
                        if (P.savedetflag & 0x1u)
                            rec[k++] = (float)((FULL && P.nextra && P.srcid <= 0) ? (detid | (S.ssrc[tid] << 16)) : detid);
                        for (unsigned i = 0; i < P.partialdata; i++) rec[k++] = S.ppath[i * B + tid];
                        if (P.savedetflag & 0x10u) { rec[k++] = px; rec[k++] = py; rec[k++] = pz; }
                        if (P.savedetflag & 0x20u) { rec[k++] = vx; rec[k++] = vy; rec[k++] = vz; }
                        // launch weight; under photon sharing MCX's slot holds the pattern pixel's
                        // index bits instead (src/mcx_core.cu:1290, 1697, 403)
                        if (P.savedetflag & 0x40u) rec[k++] = (FULL && P.srcnum > 1) ? __uint_as_float(S.spix[tid]) : S.wlaunch[tid];
                        if (FULL && P.polarized && (P.savedetflag & 0x80u)) {   // Stokes vector, 407-412
                            rec[k++] = S.stokes[tid];
                            rec[k++] = S.stokes[B + tid];
                            rec[k++] = S.stokes[2 * B + tid];
                            rec[k++] = S.stokes[3 * B + tid];
                        }
                    }
                }
            }
            S.tally[kELaunch * B + tid] += S.wlaunch[tid];
            S.tally[(detected ? kEDetect : kEEscape) * B + tid] += w;
            S.tally[kEAbsDep * B + tid] += eabs;
            S.tally[kEAbsOther * B + tid] += w0 - w;
            alive = false;
        }
    }

#undef inv_c0
#undef tw0
#undef tw1
#undef bin_a
#undef bin_b
#undef n0
#undef fnx
#undef fny
#undef fnz
#undef gscat
#undef tx0
#undef ty0
#undef tz0
#undef tx1
#undef ty1
#undef tz1

    // ---- flush: tile, tallies, counters ------------------------------------------------------
    __syncthreads();
    for (int i = tid; i < tile_elems; i += B) {
        const unsigned q = S.tile[i];
        if (q == 0u) continue;
        const float v = (float)((double)q / (double)P.d_tile_scale);
        int r = i;
        const int x = r % P.tnx; r /= P.tnx;
        const int y = r % P.tny; r /= P.tny;
        const int z = r % P.tnz; r /= P.tnz;
        const int g = r;
        const size_t addr = (size_t)((z + P.tz0) * (int)P.dimxy + (y + P.ty0) * P.nx + (x + P.tx0)) +
                            (size_t)(g + P.tg0) * P.nvox;
        field_add_large(P, addr, v);
    }
    // FP64 only here: per-thread FP32 partial sums reduced in double
    for (int k = 0; k < kNumEnergy; k++) {
        double v = (double)S.tally[k * B + tid];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
        if (lane == 0 && v != 0.0) atomicAdd(P.energy + k, v);
    }
    const unsigned c_launch = (lane == 0) ? S.wcount[3 * warp] : 0u;
    const unsigned c_tile = (lane == 0) ? S.wcount[3 * warp + 1] : 0u;
    const unsigned c_photon = (lane == 0) ? S.wcount[3 * warp + 2] : 0u;
    unsigned cnt[6] = {c_step, c_scat, c_dep, c_launch, c_photon, c_tile};
    const int cidx[6] = {kCntSteps, kCntScatter, kCntDeposit, kCntLaunch, kCntPhoton, kCntTileDeposit};
#pragma unroll
    for (int k = 0; k < 6; k++) {
        unsigned long long v = cnt[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
        if (lane == 0 && v) atomicAdd(P.counters + cidx[k], v);
    }
}

// Roofline probe: fire-and-forget FP32 reductions to addresses spread over `n` floats (a hash of
// the thread and iteration), the operation the transport kernel's deposits reduce to.
__global__ void atomic_probe_kernel(float* buf, unsigned n, int iters) {
    unsigned h = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u;
    for (int i = 0; i < iters; i++) {
        h ^= h >> 13; h *= 0x5bd1e995u; h ^= h >> 15;
        atomicAdd(buf + (h % n), 1.0f);
    }
}

// The -D R test kernel: one thread fills `out` from four seed words
// (src/mcx_core.cu:1731-1742, seeding src/mcx_rand_xorshift128p.cu:79-82).
__global__ void rng_test_kernel(const uint32_t* seeds, float* out, int n) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    unsigned long long a = ((unsigned long long)seeds[0] << 32) | seeds[1];
    unsigned long long b = ((unsigned long long)seeds[2] << 32) | seeds[3];
    for (int i = 0; i < n; i++) out[i] = rng_next(a, b);
}

__global__ void photon_stream_kernel(unsigned long long seed, unsigned long long pid, float* out, int n) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    unsigned long long a, b;
    seed_photon(seed, pid, a, b);
    for (int i = 0; i < n; i++) out[i] = rng_next(a, b);
}

// uint32 MCX voxels (bit 31 detector mask) -> one byte per voxel.
__global__ void labels_kernel(const uint32_t* __restrict__ vol, uint8_t* __restrict__ labels, size_t n,
                              unsigned int medianum, unsigned int* err) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t v = vol[i];
        const uint32_t lab = v & kMED_MASK;
        if (lab >= medianum || lab > kLabelMask) atomicOr(err, kErrBadLabel);
        labels[i] = (uint8_t)((lab & kLabelMask) | ((v & kDET_MASK) ? kLabelDet : 0u));
    }
}

// field = (field + shadow or field64) * scale, in place (src/mcx_core.cu:3687-3696 shadow merge,
// mcx_normalize src/mcx_utils.c:1227-1237 scaling; option 2 leaves negative values alone).
__global__ void merge_kernel(float* __restrict__ out, const float* __restrict__ field, const float* __restrict__ shadow,
                             const double* __restrict__ f64, size_t n, float scale, int positive_only) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = f64 ? (float)f64[i] : field[i] + (shadow ? shadow[i] : 0.f);
        if (!(positive_only && v < 0.f)) v *= scale;
        out[i] = v;
    }
}

}  // namespace

size_t transport_smem_bytes(const KParams& p, int block, bool savedet) {
    size_t b = sizeof(float4) * (size_t)p.medianum;
    b += (2 * sizeof(unsigned long long) + sizeof(int) + 3 * sizeof(unsigned)) * (size_t)(block / 32);
    b += 4 * sizeof(unsigned) * (size_t)block;
    b += sizeof(float) * kNumEnergy * (size_t)block;
    if (savedet) b += sizeof(float) * (size_t)p.partialdata * block;
    if (transport_mode(p) >= 2) b += 8 + (2 * sizeof(unsigned long long) + 12 * sizeof(float)) * (size_t)block;
    if (p.tile_on) b += sizeof(unsigned) * (size_t)p.tnx * p.tny * p.tnz * p.tng;
    return b;
}

template <bool R, bool D, int M, int K>
static const void* kernel_ptr() { return (const void*)transport_kernel<R, D, M, K>; }

static int g_minb = 4;   // register budget of the pencil variants (set by the launch tuner)

void set_transport_variant(int minb) { g_minb = (minb == 3) ? 3 : 4; }
int transport_variant() { return g_minb; }

bool transport_general(const KParams& p) { return transport_mode(p) != 0; }

int transport_mode(const KParams& p) {
    if (p.mediaformat == kMedia2LabelSplit) return 4;
    if (media_words(p.mediaformat)) return 3;
    if (p.replay || p.saveseed || p.outputtype > kOutEnergy || p.traj || p.polarized || p.saveref || p.srcnum > 1 ||
        p.nphase > 2 || p.nangle > 0 || p.nextra > 0)
        return 2;
    return (p.srctype != kSrcPencil) ? 1 : 0;
}

template <int M, int K>
static const void* pick_flags(bool reflect, bool savedet) {
    if (reflect) return savedet ? kernel_ptr<true, true, M, K>() : kernel_ptr<true, false, M, K>();
    return savedet ? kernel_ptr<false, true, M, K>() : kernel_ptr<false, false, M, K>();
}

// The pencil variants run at 4 CTAs of 256 per SM (64 registers) unless the tuner asks for 3;
// the variants with the general launch need more registers and run at 3 (80 registers).
static const void* pick(bool reflect, bool savedet, int mode) {
    if (mode == 4) return pick_flags<3, 4>(reflect, savedet);
    if (mode == 3) return pick_flags<3, 3>(reflect, savedet);
    if (mode == 2) return pick_flags<3, 2>(reflect, savedet);
    if (mode == 1) return pick_flags<3, 1>(reflect, savedet);
    return (g_minb == 3) ? pick_flags<3, 0>(reflect, savedet) : pick_flags<4, 0>(reflect, savedet);
}

int transport_blocks_per_sm(bool reflect, bool savedet, int mode, int block, size_t smem_bytes) {
    const void* k = pick(reflect, savedet, mode);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem_bytes) != cudaSuccess) return 0;
    return n;
}

void place_tile(KParams& k, int kb) {
    k.tile_on = 0;
    // area sources spread their deposits: only point sources get a tile; replay and path-length
    // outputs add other quantities than the absorbed weight the tile's scale is sized for
    if (!k.save2pt || !k.src_ok || !src_is_point(k.srctype) || k.replay || k.outputtype > kOutEnergy || k.nextra) return;
    const int elems = kb * 1024 / (int)sizeof(unsigned);
    int tg = std::min(k.maxgate, 4);
    int edge = 1;
    while ((edge + 1) * (edge + 1) * (edge + 1) * tg <= elems) edge++;
    while (edge < 6 && tg > 1) {        // prefer a deeper box over more gates
        tg--;
        edge = 1;
        while ((edge + 1) * (edge + 1) * (edge + 1) * tg <= elems) edge++;
    }
    edge = std::min(edge, std::max(k.nx, std::max(k.ny, k.nz)));
    k.tnx = std::min(edge, k.nx);
    k.tny = std::min(edge, k.ny);
    k.tnz = std::min(edge, k.nz);
    auto place = [](float c, int n, int dim) { return std::max(0, std::min(dim - n, (int)std::floor(c - 0.5f * n))); };
    // a pencil beam deposits along its direction; the other point sources all around the source
    const float ahead = (k.srctype == kSrcPencil) ? 0.5f * edge : 0.f;
    k.tx0 = place(k.src_p.x + ahead * k.src_v.x, k.tnx, k.nx);
    k.ty0 = place(k.src_p.y + ahead * k.src_v.y, k.tny, k.ny);
    k.tz0 = place(k.src_p.z + ahead * k.src_v.z, k.tnz, k.nz);
    k.tg0 = 0;
    k.tng = tg;
    k.tile_on = 1;
}

// Fill the derived block of KParams from its base fields.
static KParams finalize(const KParams& in) {
    KParams p = in;
    p.d_inv_c0 = 1.f / p.oneoverc0;
    p.d_tw0 = p.twin0 * p.d_inv_c0;
    p.d_tw1 = p.twin1 * p.d_inv_c0;
    p.d_bin_a = p.oneoverc0 * p.Rtstep;
    p.d_bin_b = p.twin0 * p.Rtstep;
    p.d_fnx = (float)p.nx; p.d_fny = (float)p.ny; p.d_fnz = (float)p.nz;
    p.d_tx0 = (float)p.tx0; p.d_ty0 = (float)p.ty0; p.d_tz0 = (float)p.tz0;
    p.d_tx1 = (float)(p.tx0 + p.tnx); p.d_ty1 = (float)(p.ty0 + p.tny); p.d_tz1 = (float)(p.tz0 + p.tnz);
    p.d_n0 = p.prop[0].w;
    p.d_gscat = (p.gscatter >= 2147483647.f) ? 2147483647 : (int)p.gscatter;
    p.d_nwork = (p.seed_mode == 1 && !p.replay) ? (unsigned long long)p.mcx_streams : p.nphoton;
    // 2^21 fixed-point units per launch weight: a deposit is at most sqrt(3) launch weights (a
    // voxel diagonal), so weight x scale stays below 2^23 as the rounding trick needs
    p.d_tile_scale = 2097152.f / fmaxf(1.f, fabsf(p.src_p.w));
    p.d_tile_flush = (float)((double)kTileFlushUnits / (double)p.d_tile_scale);
    p.d_tile_lo = p.tile_on ? (unsigned)(p.tz0 * (int)p.dimxy + p.ty0 * p.nx + p.tx0) : 0u;
    p.d_tile_span = p.tile_on ? (unsigned)((p.tnz - 1) * (int)p.dimxy + (p.tny - 1) * p.nx + p.tnx) : 0u;
    return p;
}

cudaError_t launch_transport(const KParams& in, bool reflect, bool savedet, int grid, int block, size_t smem_bytes,
                             cudaStream_t stream) {
    KParams p = finalize(in);
    // a launch of fewer than 16 photons per thread reserves nothing beyond what its dead lanes
    // need: whole-chunk reservations would leave some warps with two rounds of photons while
    // others have none, and the launch would end on their tail
    if (p.d_nwork < (unsigned long long)grid * (unsigned long long)block * 16ull) p.chunk = 1;
    const void* k = pick(reflect, savedet, transport_mode(p));
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    if (e != cudaSuccess) return e;
    void* args[] = {const_cast<KParams*>(&p)};
    return cudaLaunchKernel(k, dim3(grid), dim3(block), args, smem_bytes, stream);
}

cudaError_t launch_atomic_probe(float* buf, unsigned n, int iters, int grid, int block, cudaStream_t stream) {
    atomic_probe_kernel<<<grid, block, 0, stream>>>(buf, n, iters);
    return cudaGetLastError();
}

cudaError_t launch_rng_test(const uint32_t* d_seeds, float* d_out, int n, cudaStream_t stream) {
    rng_test_kernel<<<1, 32, 0, stream>>>(d_seeds, d_out, n);
    return cudaGetLastError();
}

cudaError_t launch_photon_stream(unsigned long long seed, unsigned long long pid, float* d_out, int n, cudaStream_t stream) {
    photon_stream_kernel<<<1, 32, 0, stream>>>(seed, pid, d_out, n);
    return cudaGetLastError();
}

cudaError_t launch_labels_from_vol(const uint32_t* d_vol, uint8_t* d_labels, size_t n, unsigned int medianum,
                                   unsigned int* d_err, cudaStream_t stream) {
    const int block = 256;
    const size_t g = (n + block - 1) / block;
    labels_kernel<<<(unsigned)(g < 4096 ? (g ? g : 1) : 4096), block, 0, stream>>>(d_vol, d_labels, n, medianum, d_err);
    return cudaGetLastError();
}

cudaError_t launch_merge_field(float* out, const float* field, const float* shadow, const double* field64, size_t n,
                               float scale, int positive_only, cudaStream_t stream) {
    const int block = 256;
    const size_t g = (n + block - 1) / block;
    merge_kernel<<<(unsigned)(g < 4096 ? (g ? g : 1) : 4096), block, 0, stream>>>(out, field, shadow, field64, n, scale, positive_only);
    return cudaGetLastError();
}

}  // namespace mcxg
