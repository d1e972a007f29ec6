// Kernels of the fluence denoiser: a 4-level 3D U-Net (16/32/64/128 channels, 3x3x3 convolutions,
// ReLU, 2x2x2 average pooling, nearest upsampling with skip concatenation, a 1x1x1 head added to
// the input log-fluence) trained on pairs of low- and high-photon fluence maps from this engine.
//
// Layout: activations are channels-last bf16, [volumes][z][y][x][channels] with x fastest over
// voxels (MCX's own voxel order, so a fluence map is used in place); convolution weights are
// bf16 [Cout][taps][Cin] with tap = dz*9 + dy*3 + dx; master weights, gradients and Adam moments
// are fp32 in the same order.
//
// Convolutions are implicit GEMMs on the BF16 tensor cores (mma.sync m16n8k16, fp32 accumulate):
//   forward   Y[v, co]  = sum_{t, ci} X[v + off(t), ci] * W[co, t, ci]      (M = voxels, N = Cout)
//   data grad dX[v, ci] = sum_{t, co} dY[v + off(t), co] * W[co, 26-t, ci] (the forward kernel run
//             on the flipped, transposed copy of W that the optimiser writes beside the weights)
//   weight gr dW[co, t, ci] = sum_v dY[v, co] * X[v + off(t), ci]         (M = Cout, N = taps*Cin,
//             K = voxels split across CTAs, fp32 atomics)
// Operand tiles are staged through a 4-deep cp.async pipeline into XOR-swizzled shared memory and
// fed to the tensor cores with ldmatrix (.trans for the weight gradient's voxel-major operands).
// Zero padding of the 3x3x3 stencil is the cp.async zero fill.  The ReLU backward is fused: a data
// gradient is multiplied by (layer input > 0) in its epilogue, so every gradient handed to a
// weight-gradient launch is already the pre-activation gradient.
#include <cuda_bf16.h>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "mcxg_denoise.h"

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 16-byte asynchronous copy global -> shared; `valid` false copies nothing and fills zeros.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void ldsm_x4(uint32_t a, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t a, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared-memory tiles are rows of CPR 16-byte chunks; chunk c of row r is stored at
// c ^ swz(r) so that the 8 rows one ldmatrix phase reads fall in 8 different bank groups.
template <int CPR>
__device__ __forceinline__ int swz(int r) {
    if constexpr (CPR >= 8) return r & 7;
    else if constexpr (CPR == 4) return (r >> 1) & 3;
    else return (r >> 2) & 1;
}

struct Geo {
    int nvol, d, h, w;
    long long m;  // voxels over all volumes
};

// Neighbour of voxel (z, y, x) at tap t of a 3x3x3 stencil (t = dz*9 + dy*3 + dx), or -1 outside.
__device__ __forceinline__ long long tap_voxel(const Geo& g, long long v, int z, int y, int x, int t, int taps) {
    if (taps == 1) return v;
    int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
    int zz = z + dz, yy = y + dy, xx = x + dx;
    if (zz < 0 || zz >= g.d || yy < 0 || yy >= g.h || xx < 0 || xx >= g.w) return -1;
    return v + (long long)dz * g.h * g.w + dy * g.w + dx;
}

// ---------------------------------------------------------------------------------------------
// Forward convolution (and data gradient): Y[v, n0:n0+BN] over a tile of BM voxels.  K runs over
// (tap, input channel) flattened, k = tap*cin + ci, in stages of BK: with few input channels one
// stage spans several taps (4 taps of 16 channels at BK = 64), so small layers still feed the
// tensor cores several k16 steps per barrier.  A chunk of 8 channels never straddles two taps
// (cin % 8 == 0); chunks past the last tap are zero-filled, as are the halo's out-of-volume rows.
template <int BM, int BN, int BK, int WARPS_M, int WARPS_N, int STAGES>
__global__ void __launch_bounds__(32 * WARPS_M * WARPS_N) conv_fwd_kernel(
    const bf16* __restrict__ x, const bf16* __restrict__ wt, const float* __restrict__ bias,
    const bf16* __restrict__ mask, bf16* __restrict__ y, Geo g, int cin, int cout, int taps, int relu) {
    constexpr int THREADS = 32 * WARPS_M * WARPS_N;
    constexpr int CPR = BK / 8;
    constexpr int WM = BM / WARPS_M, WN = BN / WARPS_N;
    constexpr int MI = WM / 16, NI = WN / 8;
    constexpr int A_ELEMS = BM * BK, B_ELEMS = BN * BK;
    constexpr int STAGE = A_ELEMS + B_ELEMS;
    constexpr int A_IT = BM * CPR / THREADS;
    static_assert(NI % 2 == 0 && MI >= 1 && A_IT >= 1 && (BM * CPR) % THREADS == 0 && THREADS % CPR == 0, "tile shape");

    extern __shared__ __align__(128) unsigned char dyn_smem[];
    bf16* sm = reinterpret_cast<bf16*>(dyn_smem);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm0 = (warp / WARPS_N) * WM, wn0 = (warp % WARPS_N) * WN;
    const long long m0 = (long long)blockIdx.x * BM;
    const int n0 = blockIdx.y * BN;
    const int ktot = taps * cin;
    const int ktiles = (ktot + BK - 1) / BK;
    const int ac = tid % CPR;                      // the A chunk column this thread loads
    const int hw = g.h * g.w;

    // packed (z, y, x) of the tile's rows, one 32-bit decomposition per row shared through shared
    // memory (-1 past the last voxel); each thread keeps those of the A rows it loads
    __shared__ int s_zyx[BM];
    {
        const int vvol = g.d * hw;
        for (int r = tid; r < BM; r += THREADS) {
            long long v = m0 + r;
            int rr = (int)(v % vvol);
            int xx = rr % g.w, q = rr / g.w;
            s_zyx[r] = v < g.m ? (((q / g.h) << 20) | ((q % g.h) << 10) | xx) : -1;
        }
    }
    __syncthreads();
    int av[A_IT], azyx[A_IT];
#pragma unroll
    for (int i = 0; i < A_IT; ++i) {
        int row = tid / CPR + i * (THREADS / CPR);
        azyx[i] = s_zyx[row];
        av[i] = azyx[i] >= 0 ? (int)(m0 + row) : -1;
    }

    auto load_stage = [&](int stage, int kt) {
        bf16* sa = sm + stage * STAGE;
        bf16* sb = sa + A_ELEMS;
        const int k = kt * BK + ac * 8;
        const int t = k / cin, ch = k - t * cin;
        int dz = 0, dy = 0, dx = 0;
        if (taps == 27) {
            dz = t / 9 - 1;
            dy = (t / 3) % 3 - 1;
            dx = t % 3 - 1;
        }
        const bool kin = t < taps;
        const int delta = dz * hw + dy * g.w + dx;
#pragma unroll
        for (int i = 0; i < A_IT; ++i) {
            int row = tid / CPR + i * (THREADS / CPR);
            int zz = (azyx[i] >> 20) + dz, yy = ((azyx[i] >> 10) & 1023) + dy, xx = (azyx[i] & 1023) + dx;
            bool ok = kin && av[i] >= 0 && zz >= 0 && zz < g.d && yy >= 0 && yy < g.h && xx >= 0 && xx < g.w;
            const bf16* p = ok ? x + (long long)(av[i] + delta) * cin + ch : x;
            cp_async16(smem_addr(sa + row * BK + ((ac ^ swz<CPR>(row)) << 3)), p, ok);
        }
#pragma unroll
        for (int i = 0; i < (BN * CPR + THREADS - 1) / THREADS; ++i) {
            int q = tid + i * THREADS;
            if (q < BN * CPR) {
                int row = q / CPR, c = q % CPR;
                int kb = kt * BK + c * 8;
                bool ok = kb < ktot;
                const bf16* p = ok ? wt + (long long)(n0 + row) * ktot + kb : wt;
                cp_async16(smem_addr(sb + row * BK + ((c ^ swz<CPR>(row)) << 3)), p, ok);
            }
        }
    };

    float acc[MI][NI][4];
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < ktiles) load_stage(s, s);
        cp_commit();
    }
    for (int kt = 0; kt < ktiles; ++kt) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        const bf16* sa = sm + (kt % STAGES) * STAGE;
        const bf16* sb = sa + A_ELEMS;
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
            uint32_t af[MI][4];
#pragma unroll
            for (int i = 0; i < MI; ++i) {
                int row = wm0 + i * 16 + (lane & 15), c = kk * 2 + (lane >> 4);
                ldsm_x4(smem_addr(sa + row * BK + ((c ^ swz<CPR>(row)) << 3)), af[i]);
            }
#pragma unroll
            for (int jj = 0; jj < NI / 2; ++jj) {
                uint32_t bfr[4];
                int row = wn0 + jj * 16 + (lane & 7) + ((lane >> 4) << 3), c = kk * 2 + ((lane >> 3) & 1);
                ldsm_x4(smem_addr(sb + row * BK + ((c ^ swz<CPR>(row)) << 3)), bfr);
#pragma unroll
                for (int i = 0; i < MI; ++i) {
                    mma_bf16(acc[i][2 * jj], af[i], bfr[0], bfr[1]);
                    mma_bf16(acc[i][2 * jj + 1], af[i], bfr[2], bfr[3]);
                }
            }
        }
        int nk = kt + STAGES - 1;
        if (nk < ktiles) load_stage(nk % STAGES, nk);
        cp_commit();
    }
    cp_wait<0>();
    __syncthreads();

    // epilogue: bias + ReLU into a padded shared tile, then 16-byte rows to global (times the mask)
    constexpr int EP = BN + 8;
    bf16* se = sm;
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j) {
            int row = wm0 + i * 16 + (lane >> 2), col = wn0 + j * 8 + (lane & 3) * 2;
            float b0 = bias ? bias[n0 + col] : 0.f, b1 = bias ? bias[n0 + col + 1] : 0.f;
            float v0 = acc[i][j][0] + b0, v1 = acc[i][j][1] + b1, v2 = acc[i][j][2] + b0, v3 = acc[i][j][3] + b1;
            if (relu) {
                v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); v2 = fmaxf(v2, 0.f); v3 = fmaxf(v3, 0.f);
            }
            *reinterpret_cast<__nv_bfloat162*>(se + row * EP + col) = __floats2bfloat162_rn(v0, v1);
            *reinterpret_cast<__nv_bfloat162*>(se + (row + 8) * EP + col) = __floats2bfloat162_rn(v2, v3);
        }
    __syncthreads();
    constexpr int CH = BN / 8;
    for (int q = tid; q < BM * CH; q += THREADS) {
        int row = q / CH, c = q % CH;
        long long v = m0 + row;
        if (v >= g.m) continue;
        uint4 val = *reinterpret_cast<const uint4*>(se + row * EP + c * 8);
        long long off = v * cout + n0 + c * 8;
        if (mask) {
            uint4 mk = *reinterpret_cast<const uint4*>(mask + off);
            uint32_t* pv = reinterpret_cast<uint32_t*>(&val);
            const uint32_t* pm = reinterpret_cast<const uint32_t*>(&mk);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                // keep each bf16 where the mask's bf16 is > 0 (sign bit clear and not +0)
                uint32_t lo = (pm[e] & 0xFFFFu), hi = pm[e] >> 16;
                uint32_t keep = ((lo & 0x8000u) == 0 && lo != 0 ? 0xFFFFu : 0u) |
                                ((hi & 0x8000u) == 0 && hi != 0 ? 0xFFFF0000u : 0u);
                pv[e] &= keep;
            }
        }
        *reinterpret_cast<uint4*>(y + off) = val;
    }
}

// ---------------------------------------------------------------------------------------------
// 3x3x3 convolution over a halo tile, for narrow outputs (BN = 16 or 32 channels): the CTA's 128
// output voxels are a 2 x 8 x 8 (z, y, x) block; for each 16-channel slice of the input it loads
// the 4 x 10 x 10 halo around that block once, and the slice's weights for all 27 taps, and forms
// every tap's A fragments by ldmatrix addressing into the halo (the 8 rows of one 8 x 8 matrix
// are 8 consecutive x of one line, i.e. 8 consecutive halo voxels).  The input is read once per
// tile instead of once per tap.  Halo and weight rows are 32 bytes (16 channels), their two
// 16-byte chunks swapped on every other group of 4 rows so the 8 rows of an ldmatrix phase fall
// in 8 different bank groups.
template <int BN>
__global__ void __launch_bounds__(128) conv3_halo_kernel(const bf16* __restrict__ x, const bf16* __restrict__ wt,
                                                         const float* __restrict__ bias,
                                                         const bf16* __restrict__ mask, bf16* __restrict__ y, Geo g,
                                                         int cin, int cout, int relu, int tiles_x, int tiles_y,
                                                         int tiles_z) {
    constexpr int TZ = 2, TY = 8, TX = 8, BM = TZ * TY * TX;
    constexpr int HZ = TZ + 2, HY = TY + 2, HX = TX + 2, HV = HZ * HY * HX;   // 400 halo voxels
    constexpr int WARPS_M = 4, WM = BM / WARPS_M, MI = WM / 16, NI = BN / 8;
    static_assert(NI % 2 == 0 && MI == 2, "tile shape");
    constexpr int ROWB = 32;                     // bytes per halo / weight row (16 channels)
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    unsigned char* sh = dyn_smem;                // [HV][32 B]
    unsigned char* sw = dyn_smem + HV * ROWB;    // [27][BN][32 B]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm0 = warp * WM;
    int tile = blockIdx.x;
    const int txi = tile % tiles_x;
    tile /= tiles_x;
    const int tyi = tile % tiles_y;
    tile /= tiles_y;
    const int tzi = tile % tiles_z;
    const int n = tile / tiles_z;
    const int x0 = txi * TX, y0 = tyi * TY, z0 = tzi * TZ;
    const int n0 = blockIdx.y * BN;
    const long long vol0 = (long long)n * g.d * g.h * g.w;

    // halo-voxel index of this lane's A rows (tap offset added per tap)
    int hbase[MI];
#pragma unroll
    for (int i = 0; i < MI; ++i) {
        int r = wm0 + i * 16 + (lane & 15);
        int tx = r & 7, ty = (r >> 3) & 7, tz = r >> 6;
        hbase[i] = ((tz + 1) * HY + (ty + 1)) * HX + (tx + 1);
    }
    const int achunk = lane >> 4;                // A: lanes 16-31 read the second 8 channels

    float acc[MI][NI][4];
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

    const int slices = cin / 16;
    for (int sl = 0; sl < slices; ++sl) {
        const int c0 = sl * 16;
        // halo: HV rows x 2 chunks, zero outside the volume
        for (int q = tid; q < HV * 2; q += 128) {
            int hv = q >> 1, c = q & 1;
            int hx = hv % HX, hy = (hv / HX) % HY, hz = hv / (HX * HY);
            int zz = z0 + hz - 1, yy = y0 + hy - 1, xx = x0 + hx - 1;
            bool ok = zz >= 0 && zz < g.d && yy >= 0 && yy < g.h && xx >= 0 && xx < g.w;
            const bf16* p = ok ? x + (vol0 + ((long long)zz * g.h + yy) * g.w + xx) * cin + c0 + c * 8 : x;
            cp_async16(smem_addr(sh + hv * ROWB + ((c ^ ((hv >> 2) & 1)) << 4)), p, ok);
        }
        // weights of this slice for all taps: row (t, co), 16 channels
        for (int q = tid; q < 27 * BN * 2; q += 128) {
            int row = q >> 1, c = q & 1;
            int t = row / BN, co = row - t * BN;
            const bf16* p = wt + ((long long)(n0 + co) * 27 + t) * cin + c0 + c * 8;
            cp_async16(smem_addr(sw + row * ROWB + ((c ^ ((row >> 2) & 1)) << 4)), p, true);
        }
        cp_commit();
        cp_wait<0>();
        __syncthreads();
#pragma unroll 3
        for (int t = 0; t < 27; ++t) {
            const int off = (t / 9 - 1) * (HY * HX) + ((t / 3) % 3 - 1) * HX + (t % 3 - 1);
            uint32_t af[MI][4];
#pragma unroll
            for (int i = 0; i < MI; ++i) {
                int hv = hbase[i] + off;
                ldsm_x4(smem_addr(sh + hv * ROWB + ((achunk ^ ((hv >> 2) & 1)) << 4)), af[i]);
            }
#pragma unroll
            for (int jj = 0; jj < NI / 2; ++jj) {
                uint32_t bfr[4];
                int row = t * BN + jj * 16 + (lane & 7) + ((lane >> 4) << 3);
                int c = (lane >> 3) & 1;
                ldsm_x4(smem_addr(sw + row * ROWB + ((c ^ ((row >> 2) & 1)) << 4)), bfr);
#pragma unroll
                for (int i = 0; i < MI; ++i) {
                    mma_bf16(acc[i][2 * jj], af[i], bfr[0], bfr[1]);
                    mma_bf16(acc[i][2 * jj + 1], af[i], bfr[2], bfr[3]);
                }
            }
        }
        __syncthreads();                 // the next slice overwrites the halo and the weights
    }

    // epilogue: bias + ReLU into a padded shared tile, then 16-byte rows to global (times the mask)
    constexpr int EP = BN + 8;
    bf16* se = reinterpret_cast<bf16*>(dyn_smem);
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j) {
            int row = wm0 + i * 16 + (lane >> 2), col = j * 8 + (lane & 3) * 2;
            float b0 = bias ? bias[n0 + col] : 0.f, b1 = bias ? bias[n0 + col + 1] : 0.f;
            float v0 = acc[i][j][0] + b0, v1 = acc[i][j][1] + b1, v2 = acc[i][j][2] + b0, v3 = acc[i][j][3] + b1;
            if (relu) {
                v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); v2 = fmaxf(v2, 0.f); v3 = fmaxf(v3, 0.f);
            }
            *reinterpret_cast<__nv_bfloat162*>(se + row * EP + col) = __floats2bfloat162_rn(v0, v1);
            *reinterpret_cast<__nv_bfloat162*>(se + (row + 8) * EP + col) = __floats2bfloat162_rn(v2, v3);
        }
    __syncthreads();
    constexpr int CH = BN / 8;
    for (int q = tid; q < BM * CH; q += 128) {
        int r = q / CH, c = q % CH;
        int xx = x0 + (r & 7), yy = y0 + ((r >> 3) & 7), zz = z0 + (r >> 6);
        if (xx >= g.w || yy >= g.h || zz >= g.d) continue;
        long long v = vol0 + ((long long)zz * g.h + yy) * g.w + xx;
        uint4 val = *reinterpret_cast<const uint4*>(se + r * EP + c * 8);
        long long o = v * cout + n0 + c * 8;
        if (mask) {
            uint4 mk = *reinterpret_cast<const uint4*>(mask + o);
            uint32_t* pv = reinterpret_cast<uint32_t*>(&val);
            const uint32_t* pm = reinterpret_cast<const uint32_t*>(&mk);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                uint32_t lo = (pm[e] & 0xFFFFu), hi = pm[e] >> 16;
                uint32_t keep = ((lo & 0x8000u) == 0 && lo != 0 ? 0xFFFFu : 0u) |
                                ((hi & 0x8000u) == 0 && hi != 0 ? 0xFFFF0000u : 0u);
                pv[e] &= keep;
            }
        }
        *reinterpret_cast<uint4*>(y + o) = val;
    }
}

// ---------------------------------------------------------------------------------------------
// 3x3x3 convolution for narrow outputs (BN = 16 or 32 channels) on the fifth-generation tensor
// cores: tcgen05.mma (cta_group::1, kind::f16, BF16 operands from shared memory, FP32 accumulator
// in tensor memory), issued by one thread, with the input halos brought in by TMA.  A tile is two
// z-planes of 16 y rows x 8 x voxels; each plane is one M = 128 MMA, whose eight-voxel rows are
// a uniform stride apart in the halo.  Per 16-channel slice of the input, the 4 x 18 x 10 halo
// around the tile lands as two 8-channel planes of 16-byte rows, and every tap's A operand is the same halo
// seen through a descriptor whose start moves by the tap's row offset: K-major, no swizzle, core
// matrices of 8 consecutive rows (8 consecutive x), the 8-row groups HX rows apart (stride byte
// offset), the second 8 channels one plane further on (leading byte offset).  The weights of a
// slice's 27 taps sit in shared memory as [tap][8-channel half][co] 16-byte rows.  Each slice is
// 27 MMAs of 128 x BN x 16 into one accumulator.  The epilogue reads the accumulator rows (TMEM
// lane = voxel) with tcgen05.ld, adds bias, applies ReLU and the mask, and stores bf16.  Every
// wait is bounded: a wait that gives up sets g_dn_fault, and the CTA still releases its tensor
// memory and returns.
__device__ unsigned g_dn_fault;

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

// Waits for the completion of the mbarrier phase of parity `parity`; false after about a second.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > 2000000000LL) return false;
    }
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

template <int BN>
struct TcConvShape {
    static constexpr int TZ = 2, TY = 16, TX = 8;                         // two z-planes of 128 voxels
    static constexpr int HZ = TZ + 2, HY = TY + 2, HX = TX + 2, HV = HZ * HY * HX;   // 720 halo rows
    static constexpr int PLANE = HV * 16;                                 // 11520 B, a multiple of 128
    static constexpr int HALO = 2 * PLANE;                                // one stage: 16 channels
    static constexpr int HALO_BYTES = 2 * HV * 16;                        // bytes the two copies bring
    static constexpr int WTAP = 2 * BN * 16;                              // one tap's weights
    static constexpr int WSLICE = 27 * WTAP;                              // one 16-channel slice
    static constexpr int MAX_STAGES = 4;
};

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

// Warp roles: warps 0-3 drain the accumulators (warp w reads TMEM lanes 32w..32w+31, the voxels of
// its quarter of the tile), warp 4 issues the TMA copies of the halos, warp 5 issues the MMAs.
// The CTA is persistent: it loads the weights of every input slice once, then walks its tiles
// (blockIdx.x, + gridDim.x, ...) as a sequence of (tile, slice) items.  Each item is one halo: two
// TMA tile copies (channels c..c+7 and c+8..c+15) of a 4 x 18 x 10 voxel box of the channels-last
// activations, described by a 5-D tensor map (channel, x, y, z, volume) whose out-of-volume rows
// arrive as zeros; the box lands as 720 rows of 16 bytes, x fastest, which is the A operand's
// canonical no-swizzle K-major layout.  Halos cycle through `stages` buffers (full barriers: the
// copies landed; empty barriers: the MMAs that read the buffer finished), and tiles through two
// TMEM accumulators (accfull: a tile's MMAs finished; accempty: its epilogue has read it), so
// copies, MMAs and epilogues of neighbouring items overlap.
template <int BN>
__global__ void __launch_bounds__(192) conv3_tc_kernel(const __grid_constant__ CUtensorMap tmap,
                                                       const bf16* __restrict__ wt, const float* __restrict__ bias,
                                                       const bf16* __restrict__ mask, bf16* __restrict__ y, Geo g,
                                                       int cin, int cout, int relu, int tiles_x, int tiles_y,
                                                       int ntiles, int stages) {
    using S = TcConvShape<BN>;
    constexpr uint32_t TMEM_COLS = 4 * BN;          // two tiles in flight x two z-planes of BN columns
    static_assert(BN == 16 || BN == 32, "tile width");
    static_assert(S::WSLICE % 128 == 0 && S::PLANE % 128 == 0 && S::PLANE >= S::HV * 16, "TMA / UMMA alignment");
    extern __shared__ __align__(1024) unsigned char dyn_smem[];
    __shared__ __align__(8) uint64_t s_bar[2 * S::MAX_STAGES + 4];
    __shared__ uint32_t s_tmem;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int slices = cin / 16;
    const int n0 = blockIdx.y * BN;
    // weights first, then the halo stages (the weight block is a multiple of 128 bytes)
    const uint32_t sw_addr = smem_addr(dyn_smem);
    const uint32_t sh_addr = sw_addr + slices * S::WSLICE;
    const uint32_t full0 = smem_addr(&s_bar[0]), empty0 = full0 + 8 * S::MAX_STAGES;
    const uint32_t accfull0 = empty0 + 8 * S::MAX_STAGES, accempty0 = accfull0 + 16;
    const int my_tiles = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int items = my_tiles * slices;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&s_tmem)),
                     "n"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int i = 0; i < 2 * S::MAX_STAGES + 2; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(full0 + 8 * i));
        for (int i = 0; i < 2; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(accempty0 + 8 * i));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // the weights of every slice, once: [slice][tap][8-channel half][co] rows of 16 bytes
    for (int q = tid; q < slices * 27 * 2 * BN; q += 192) {
        const int co = q % BN, r = q / BN, kb = r & 1, t = (r >> 1) % 27, sl = (r >> 1) / 27;
        const bf16* p = wt + ((long long)(n0 + co) * 27 + t) * cin + sl * 16 + kb * 8;
        cp_async16(sw_addr + sl * S::WSLICE + t * S::WTAP + kb * BN * 16 + co * 16, p, true);
    }
    cp_commit();
    cp_wait<0>();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;

    struct TileAt {
        int x0, y0, z0, n;
    };
    auto tile_at = [&](int j) {
        int tile = (int)blockIdx.x + j * (int)gridDim.x;
        TileAt r;
        r.x0 = (tile % tiles_x) * S::TX;
        tile /= tiles_x;
        r.y0 = (tile % tiles_y) * S::TY;
        tile /= tiles_y;
        const int tz = (g.d + S::TZ - 1) / S::TZ;
        r.z0 = (tile % tz) * S::TZ;
        r.n = tile / tz;
        return r;
    };

    bool fault = false;
    if (warp == 4) {
        // ---- producer: TMA halo copies ----------------------------------------------------------
        if (lane == 0) {
            const uint64_t map = reinterpret_cast<uint64_t>(&tmap);
            for (int k = 0; k < items; ++k) {
                const int b = k % stages;
                if (k >= stages && !mbar_wait(empty0 + 8 * b, ((k / stages) - 1) & 1)) {
                    fault = true;
                    break;
                }
                const TileAt T = tile_at(k / slices);
                const int c0 = (k % slices) * 16;
                const uint32_t bar = full0 + 8 * b, dst = sh_addr + b * S::HALO;
                mbar_expect_tx(bar, S::HALO_BYTES);
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    asm volatile(
                        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
                        "%5, %6}], [%7];\n" ::"r"(dst + h * S::PLANE),
                        "l"(map), "r"(c0 + 8 * h), "r"(T.x0 - 1), "r"(T.y0 - 1), "r"(T.z0 - 1), "r"(T.n), "r"(bar)
                        : "memory");
            }
        }
        __syncwarp();
    } else if (warp == 5) {
        // ---- MMA issue: one thread --------------------------------------------------------------
        if (lane == 0) {
            for (int k = 0; k < items; ++k) {
                const int j = k / slices, sl = k - j * slices, b = k % stages;
                if (!mbar_wait(full0 + 8 * b, (k / stages) & 1)) {
                    fault = true;
                    break;
                }
                if (sl == 0 && j >= 2 && !mbar_wait(accempty0 + 8 * (j & 1), ((j - 2) >> 1) & 1)) {
                    fault = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = tmem + (uint32_t)((j & 1) * 2 * BN);
                // descriptors of tap 0; a tap (and the second z-plane, one halo plane further on)
                // moves the start address (bits 0-13, in 16-byte units) by a constant, so the 54 MMAs
                // issue back to back; both planes share the tap's weights
                const uint64_t ad0 = umma_desc(sh_addr + b * S::HALO, S::PLANE, S::HX * 16);
                const uint64_t bd0 = umma_desc(sw_addr + sl * S::WSLICE, BN * 16, 128);
#pragma unroll
                for (int t = 0; t < 27; ++t) {
                    const uint64_t bd = bd0 + (uint64_t)(t * S::WTAP >> 4);
                    const uint32_t accum = (sl > 0 || t > 0) ? 1u : 0u;
#pragma unroll
                    for (int zp = 0; zp < S::TZ; ++zp) {
                        const uint64_t ad =
                            ad0 + (uint64_t)((((t / 9 + zp) * S::HY + (t / 3) % 3) * S::HX + t % 3) * 16 >> 4);
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d + zp * BN),
                            "l"(ad), "l"(bd), "n"(umma_idesc_bf16(BN)), "r"(accum)
                            : "memory");
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 empty0 + 8 * b)
                             : "memory");
                if (sl == slices - 1)
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     accfull0 + 8 * (j & 1))
                                 : "memory");
            }
        }
        __syncwarp();
    } else {
        // ---- epilogue: warps 0-3 -------------------------------------------------------------------
        for (int j = 0; j < my_tiles; ++j) {
            const bool ok = mbar_wait(accfull0 + 8 * (j & 1), (j >> 1) & 1);
            if (!__all_sync(0xffffffffu, ok)) {
                fault = true;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const TileAt T = tile_at(j);
            const int r = warp * 32 + lane;             // accumulator row = TMEM lane = voxel of a plane
            const int yy = T.y0 + (r >> 3), xx = T.x0 + (r & 7);
            uint32_t v[S::TZ][BN];
#pragma unroll
            for (int zp = 0; zp < S::TZ; ++zp)
#pragma unroll
                for (int c0 = 0; c0 < BN; c0 += 16)
                    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((j & 1) * 2 * BN + zp * BN + c0),
                              *reinterpret_cast<uint32_t(*)[16]>(&v[zp][c0]));
            // the accumulators are free again once every lane of the four warps has read them
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(accempty0 + 8 * (j & 1));
#pragma unroll
            for (int zp = 0; zp < S::TZ; ++zp) {
                if (yy >= g.h || xx >= g.w || T.z0 + zp >= g.d) continue;
                const long long vo = (((long long)T.n * g.d + T.z0 + zp) * g.h + yy) * g.w + xx;
#pragma unroll
                for (int c0 = 0; c0 < BN; c0 += 16) {
                    uint32_t pk[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        float a = __uint_as_float(v[zp][c0 + 2 * e]), bb = __uint_as_float(v[zp][c0 + 2 * e + 1]);
                        if (bias) {
                            a += bias[n0 + c0 + 2 * e];
                            bb += bias[n0 + c0 + 2 * e + 1];
                        }
                        if (relu) {
                            a = fmaxf(a, 0.f);
                            bb = fmaxf(bb, 0.f);
                        }
                        __nv_bfloat162 h2 = __floats2bfloat162_rn(a, bb);
                        pk[e] = *reinterpret_cast<uint32_t*>(&h2);
                    }
                    const long long o = vo * cout + n0 + c0;
#pragma unroll
                    for (int hlf = 0; hlf < 2; ++hlf) {
                        uint4 val = make_uint4(pk[4 * hlf], pk[4 * hlf + 1], pk[4 * hlf + 2], pk[4 * hlf + 3]);
                        if (mask) {
                            uint4 mk = *reinterpret_cast<const uint4*>(mask + o + 8 * hlf);
                            uint32_t* pv = reinterpret_cast<uint32_t*>(&val);
                            const uint32_t* pm = reinterpret_cast<const uint32_t*>(&mk);
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                uint32_t lo = (pm[e] & 0xFFFFu), hi = pm[e] >> 16;
                                uint32_t keep = ((lo & 0x8000u) == 0 && lo != 0 ? 0xFFFFu : 0u) |
                                                ((hi & 0x8000u) == 0 && hi != 0 ? 0xFFFF0000u : 0u);
                                pv[e] &= keep;
                            }
                        }
                        *reinterpret_cast<uint4*>(y + o + 8 * hlf) = val;
                    }
                }
            }
        }
    }
    if (fault && lane == 0) atomicOr(&g_dn_fault, 1u);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "n"(TMEM_COLS));
}

// ---------------------------------------------------------------------------------------------
// Weight gradient: dW[co, n] += sum_v dY[v, co] * X[v + off(t), ci], n = t*Cin + ci, over the
// voxel slice [blockIdx.y*kslice, +kslice).  BM = Cout (the whole output-channel range), BN = 64
// columns of (tap, ci); 128 threads; K staged 32 voxels at a time.
template <int BM, int STAGES>
__global__ void __launch_bounds__(128) conv_wgrad_kernel(const bf16* __restrict__ dy, const bf16* __restrict__ x,
                                                         float* __restrict__ dw, Geo g, int cin, int taps,
                                                         long long kslice) {
    constexpr int BN = 64, BK = 32;
    constexpr int CPA = BM / 8, CPB = BN / 8;
    constexpr int WARPS_M = BM >= 32 ? 2 : 1;
    constexpr int WARPS_N = 4 / WARPS_M;
    constexpr int WM = BM / WARPS_M, WN = BN / WARPS_N;
    constexpr int MI = WM / 16, NI = WN / 8;
    constexpr int A_ELEMS = BK * BM, B_ELEMS = BK * BN;
    constexpr int STAGE = A_ELEMS + B_ELEMS;
    static_assert(NI % 2 == 0 && MI >= 1, "tile shape");

    extern __shared__ __align__(128) unsigned char dyn_smem[];
    bf16* sm = reinterpret_cast<bf16*>(dyn_smem);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm0 = (warp / WARPS_N) * WM, wn0 = (warp % WARPS_N) * WN;
    const int ntot = taps * cin;
    const int nt0 = blockIdx.x * BN;
    const long long kbeg = (long long)blockIdx.y * kslice;
    const long long kend = min(g.m, kbeg + kslice);
    if (kbeg >= kend) return;
    const int ktiles = (int)((kend - kbeg + BK - 1) / BK);
    const long long vvol = (long long)g.d * g.h * g.w;

    // the B (input) chunks this thread loads: one fixed column chunk (tap, 8 channels) and rows
    // tid / CPB + 16 i, whose voxel coordinates advance by BK voxels per stage (stages are
    // loaded in order), so no division runs inside the K loop
    constexpr int B_IT = BK * CPB / 128;
    static_assert(B_IT * 128 == BK * CPB && 128 % CPB == 0, "B loader shape");
    const int bc = tid % CPB;
    const int ncol = nt0 + bc * 8;
    const bool col_ok = ncol < ntot;
    const int tap = col_ok ? ncol / cin : 0, ci = col_ok ? ncol - tap * cin : 0;
    int tz = 0, ty = 0, tx = 0;
    if (taps == 27) {
        tz = tap / 9 - 1;
        ty = (tap / 3) % 3 - 1;
        tx = tap % 3 - 1;
    }
    const long long delta = (long long)tz * g.h * g.w + ty * g.w + tx;
    long long bv[B_IT];
    int bz[B_IT], by[B_IT], bx[B_IT];
#pragma unroll
    for (int i = 0; i < B_IT; ++i) {
        bv[i] = kbeg + tid / CPB + i * (128 / CPB);
        long long r = bv[i] % vvol;
        bx[i] = (int)(r % g.w);
        by[i] = (int)((r / g.w) % g.h);
        bz[i] = (int)(r / ((long long)g.w * g.h));
    }

    auto load_stage = [&](int stage, int kt) {
        bf16* sa = sm + stage * STAGE;
        bf16* sb = sa + A_ELEMS;
        const long long vb = kbeg + (long long)kt * BK;
        for (int q = tid; q < BK * CPA; q += 128) {
            int row = q / CPA, c = q % CPA;
            long long v = vb + row;
            bool ok = v < kend;
            const bf16* p = ok ? dy + v * BM + c * 8 : dy;
            cp_async16(smem_addr(sa + row * BM + ((c ^ swz<CPA>(row)) << 3)), p, ok);
        }
#pragma unroll
        for (int i = 0; i < B_IT; ++i) {
            int row = tid / CPB + i * (128 / CPB);
            int zz = bz[i] + tz, yy = by[i] + ty, xx = bx[i] + tx;
            bool ok = col_ok && bv[i] < kend && zz >= 0 && zz < g.d && yy >= 0 && yy < g.h && xx >= 0 && xx < g.w;
            const bf16* p = ok ? x + (bv[i] + delta) * cin + ci : x;
            cp_async16(smem_addr(sb + row * BN + ((bc ^ swz<CPB>(row)) << 3)), p, ok);
            // next stage: BK voxels further on
            bv[i] += BK;
            bx[i] += BK;
            while (bx[i] >= g.w) {
                bx[i] -= g.w;
                if (++by[i] >= g.h) {
                    by[i] = 0;
                    if (++bz[i] >= g.d) bz[i] = 0;
                }
            }
        }
    };

    float acc[MI][NI][4];
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < ktiles) load_stage(s, s);
        cp_commit();
    }
    for (int kt = 0; kt < ktiles; ++kt) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        const bf16* sa = sm + (kt % STAGES) * STAGE;
        const bf16* sb = sa + A_ELEMS;
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
            const int qm = lane >> 3, r8 = lane & 7;
            uint32_t af[MI][4];
#pragma unroll
            for (int i = 0; i < MI; ++i) {
                int row = kk * 16 + r8 + ((qm >> 1) << 3);
                int c = (wm0 + i * 16) / 8 + (qm & 1);
                ldsm_x4_t(smem_addr(sa + row * BM + ((c ^ swz<CPA>(row)) << 3)), af[i]);
            }
#pragma unroll
            for (int jj = 0; jj < NI / 2; ++jj) {
                uint32_t bfr[4];
                int row = kk * 16 + r8 + ((qm & 1) << 3);
                int c = (wn0 + jj * 16) / 8 + (qm >> 1);
                ldsm_x4_t(smem_addr(sb + row * BN + ((c ^ swz<CPB>(row)) << 3)), bfr);
#pragma unroll
                for (int i = 0; i < MI; ++i) {
                    mma_bf16(acc[i][2 * jj], af[i], bfr[0], bfr[1]);
                    mma_bf16(acc[i][2 * jj + 1], af[i], bfr[2], bfr[3]);
                }
            }
        }
        int nk = kt + STAGES - 1;
        if (nk < ktiles) load_stage(nk % STAGES, nk);
        cp_commit();
    }
    cp_wait<0>();

#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NI; ++j) {
            int co = wm0 + i * 16 + (lane >> 2);
            int n = nt0 + wn0 + j * 8 + (lane & 3) * 2;
            if (n < ntot) {
                atomicAdd(dw + (long long)co * ntot + n, acc[i][j][0]);
                atomicAdd(dw + (long long)(co + 8) * ntot + n, acc[i][j][2]);
            }
            if (n + 1 < ntot) {
                atomicAdd(dw + (long long)co * ntot + n + 1, acc[i][j][1]);
                atomicAdd(dw + (long long)(co + 8) * ntot + n + 1, acc[i][j][3]);
            }
        }
}

// db[c] += sum_v dY[v, c]
__global__ void bias_grad_kernel(const bf16* __restrict__ dy, float* __restrict__ db, long long m, int c,
                                 long long rows_per_block) {
    const int lanes = blockDim.x / c;  // rows processed side by side
    const int ch = threadIdx.x % c, r0 = threadIdx.x / c;
    long long beg = blockIdx.x * rows_per_block, end = min(m, beg + rows_per_block);
    float s = 0.f;
    for (long long v = beg + r0; v < end; v += lanes) s += __bfloat162float(dy[v * c + ch]);
    atomicAdd(db + ch, s);
}

__device__ __forceinline__ void load8(const bf16* p, float (&f)[8]) {
    uint4 u = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float2 t = __bfloat1622float2(h[e]);
        f[2 * e] = t.x;
        f[2 * e + 1] = t.y;
    }
}
__device__ __forceinline__ void store8(bf16* p, const float (&f)[8]) {
    uint4 u;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
    for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(f[2 * e], f[2 * e + 1]);
    *reinterpret_cast<uint4*>(p) = u;
}

// 2x2x2 average pooling; (d, h, w) are the fine grid's sizes.  One thread per coarse voxel and
// 8-channel chunk.
__global__ void pool_kernel(const bf16* __restrict__ x, bf16* __restrict__ y, int nvol, int d, int h, int w, int c) {
    const int d2 = d / 2, h2 = h / 2, w2 = w / 2, cc = c / 8;
    long long total = (long long)nvol * d2 * h2 * w2 * cc;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        int ch = (int)(q % cc);
        long long v = q / cc;
        int xx = (int)(v % w2), yy = (int)((v / w2) % h2), zz = (int)((v / ((long long)w2 * h2)) % d2);
        long long n = v / ((long long)w2 * h2 * d2);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 8; ++k) {
            long long fv = ((n * d + 2 * zz + (k >> 2)) * h + 2 * yy + ((k >> 1) & 1)) * w + 2 * xx + (k & 1);
            float f[8];
            load8(x + fv * c + ch * 8, f);
#pragma unroll
            for (int e = 0; e < 8; ++e) s[e] += f[e];
        }
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] *= 0.125f;
        store8(y + v * c + ch * 8, s);
    }
}

// cat[v, 0:c1] = low[parent(v)], cat[v, c1:c1+c2] = skip[v]; (d, h, w) fine sizes.
__global__ void upcat_kernel(const bf16* __restrict__ low, const bf16* __restrict__ skip, bf16* __restrict__ cat,
                             int nvol, int d, int h, int w, int c1, int c2) {
    const int ct = (c1 + c2) / 8;
    long long total = (long long)nvol * d * h * w * ct;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        int ch = (int)(q % ct);
        long long v = q / ct;
        const bf16* src;
        if (ch * 8 < c1) {
            int xx = (int)(v % w), yy = (int)((v / w) % h), zz = (int)((v / ((long long)w * h)) % d);
            long long n = v / ((long long)w * h * d);
            long long pv = ((n * (d / 2) + zz / 2) * (h / 2) + yy / 2) * (w / 2) + xx / 2;
            src = low + pv * c1 + ch * 8;
        } else {
            src = skip + v * c2 + (ch * 8 - c1);
        }
        *reinterpret_cast<uint4*>(cat + v * (c1 + c2) + ch * 8) = *reinterpret_cast<const uint4*>(src);
    }
}

// dlow[u, c] = (sum over the 8 children of dcat[child, c]) * (low[u, c] > 0), c < c1.
__global__ void upcat_bwd_kernel(const bf16* __restrict__ dcat, const bf16* __restrict__ low, bf16* __restrict__ dlow,
                                 int nvol, int d, int h, int w, int c1, int c2) {
    const int d2 = d / 2, h2 = h / 2, w2 = w / 2, cc = c1 / 8, ct = c1 + c2;
    long long total = (long long)nvol * d2 * h2 * w2 * cc;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        int ch = (int)(q % cc);
        long long u = q / cc;
        int xx = (int)(u % w2), yy = (int)((u / w2) % h2), zz = (int)((u / ((long long)w2 * h2)) % d2);
        long long n = u / ((long long)w2 * h2 * d2);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 8; ++k) {
            long long fv = ((n * d + 2 * zz + (k >> 2)) * h + 2 * yy + ((k >> 1) & 1)) * w + 2 * xx + (k & 1);
            float f[8];
            load8(dcat + fv * ct + ch * 8, f);
#pragma unroll
            for (int e = 0; e < 8; ++e) s[e] += f[e];
        }
        float lv[8];
        load8(low + u * c1 + ch * 8, lv);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] = lv[e] > 0.f ? s[e] : 0.f;
        store8(dlow + u * c1 + ch * 8, s);
    }
}

// denc[v, c] = (dpool[parent(v), c] / 8 + dcat[v, c1 + c]) * (enc[v, c] > 0); dcat may be null
// (no skip path).  (d, h, w) fine sizes; c = encoder channels.
__global__ void unpool_add_kernel(const bf16* __restrict__ dpool, const bf16* __restrict__ dcat,
                                  const bf16* __restrict__ enc, bf16* __restrict__ denc, int nvol, int d, int h, int w,
                                  int c1, int c) {
    const int cc = c / 8;
    long long total = (long long)nvol * d * h * w * cc;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        int ch = (int)(q % cc);
        long long v = q / cc;
        int xx = (int)(v % w), yy = (int)((v / w) % h), zz = (int)((v / ((long long)w * h)) % d);
        long long n = v / ((long long)w * h * d);
        long long pv = ((n * (d / 2) + zz / 2) * (h / 2) + yy / 2) * (w / 2) + xx / 2;
        float a[8], b[8], e8[8];
        load8(dpool + pv * c + ch * 8, a);
        if (dcat) load8(dcat + v * (c1 + c) + c1 + ch * 8, b);
        else
            for (int e = 0; e < 8; ++e) b[e] = 0.f;
        load8(enc + v * c + ch * 8, e8);
        float o[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) o[e] = e8[e] > 0.f ? a[e] * 0.125f + b[e] : 0.f;
        store8(denc + v * c + ch * 8, o);
    }
}

// Head: out[v] = xres[v] + b + sum_c w[c] * act[v, c] (16 channels).  With a target, also the
// masked L1 loss, dact = g * w * (act > 0), dw += g * act, db += g, g = sign(out - t) * valid * inv.
__global__ void __launch_bounds__(256) head_kernel(const bf16* __restrict__ act, const float* __restrict__ xres,
                                                   const float* __restrict__ w, const float* __restrict__ b,
                                                   const float* __restrict__ target, const float* __restrict__ valid,
                                                   float* __restrict__ out, bf16* __restrict__ dact,
                                                   float* __restrict__ dw, float* __restrict__ db,
                                                   float* __restrict__ loss, long long m, float inv) {
    __shared__ float red[8][18];
    float gw[16], gb = 0.f, ls = 0.f;
#pragma unroll
    for (int c = 0; c < 16; ++c) gw[c] = 0.f;
    float wc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) wc[c] = w[c];
    const float bias = b[0];
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < m; v += (long long)gridDim.x * blockDim.x) {
        float a[16];
        float lo[8], hi[8];
        load8(act + v * 16, lo);
        load8(act + v * 16 + 8, hi);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            a[e] = lo[e];
            a[8 + e] = hi[e];
        }
        float o = xres[v] + bias;
#pragma unroll
        for (int c = 0; c < 16; ++c) o = fmaf(wc[c], a[c], o);
        if (out) out[v] = o;
        if (target) {
            float diff = o - target[v], vl = valid[v];
            ls += fabsf(diff) * vl;
            float gr = (diff > 0.f ? 1.f : (diff < 0.f ? -1.f : 0.f)) * vl * inv;
            gb += gr;
#pragma unroll
            for (int c = 0; c < 16; ++c) gw[c] += gr * a[c];
            float da[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) da[c] = a[c] > 0.f ? gr * wc[c] : 0.f;
            float d0[8], d1[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                d0[e] = da[e];
                d1[e] = da[8 + e];
            }
            store8(dact + v * 16, d0);
            store8(dact + v * 16 + 8, d1);
        }
    }
    if (!target) return;
    // block reduction of the 18 sums (16 weights, bias, loss)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float vals[18];
#pragma unroll
    for (int c = 0; c < 16; ++c) vals[c] = gw[c];
    vals[16] = gb;
    vals[17] = ls;
#pragma unroll
    for (int k = 0; k < 18; ++k) {
        float s = vals[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[warp][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < 18) {
        float s = 0.f;
        for (int k = 0; k < (int)(blockDim.x / 32); ++k) s += red[k][threadIdx.x];
        if (threadIdx.x < 16) atomicAdd(dw + threadIdx.x, s);
        else if (threadIdx.x == 16) atomicAdd(db, s);
        else atomicAdd(loss, s);
    }
}

// Input features of one voxel (16 channels, 0..6 used), with l0, l3, l5 = log10(m + 1e-10) of the
// noisy fluence F and of its means over the in-bounds voxels of the 3x3x3 and 5x5x5
// neighbourhoods:
//   0: (l3 + 5) / 3      1: clamp(4 (l0 - l3), -4, 4)      2: clamp(4 (l5 - l3), -4, 4)
//   3: 1 where F is 0    4: log10(mua) + 2    5: log10(mus (1 - g))    6: (log10(photons) - 5.5) * 2
// and xres[v] = l3, the residual base the head adds its correction to.  The means are taken in
// linear fluence, where a voxel no photon reached is a zero among its neighbours rather than a
// -10 outlier as in log space; channels 1 and 2 hand the network the noise and the curvature at
// the scale of its correction instead of as small differences of large inputs.
__global__ void pack_kernel(const float* __restrict__ flux, const uint8_t* __restrict__ label,
                            const float* __restrict__ props, const float* __restrict__ log_photons,
                            bf16* __restrict__ x0, float* __restrict__ xres, Geo g, int nprop) {
    const long long vvol = (long long)g.d * g.h * g.w;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < g.m; v += (long long)gridDim.x * blockDim.x) {
        int n = (int)(v / vvol);
        long long r = v % vvol;
        int x = (int)(r % g.w), y = (int)((r / g.w) % g.h), z = (int)(r / ((long long)g.w * g.h));
        float s3 = 0.f, s5 = 0.f;
        int c3 = 0, c5 = 0;
        for (int dz = -2; dz <= 2; ++dz) {
            int zz = z + dz;
            if (zz < 0 || zz >= g.d) continue;
            for (int dy = -2; dy <= 2; ++dy) {
                int yy = y + dy;
                if (yy < 0 || yy >= g.h) continue;
                const float* row = flux + ((long long)n * vvol + ((long long)zz * g.h + yy) * g.w);
                bool inner = dz >= -1 && dz <= 1 && dy >= -1 && dy <= 1;
                for (int dx = -2; dx <= 2; ++dx) {
                    int xx = x + dx;
                    if (xx < 0 || xx >= g.w) continue;
                    float f = fmaxf(row[xx], 0.f);
                    s5 += f;
                    ++c5;
                    if (inner && dx >= -1 && dx <= 1) {
                        s3 += f;
                        ++c3;
                    }
                }
            }
        }
        int lab = label[v];
        if (lab >= nprop) lab = nprop - 1;
        const float* pr = props + ((long long)n * nprop + lab) * 4;
        const float fv = flux[v];
        float l0 = log10f(fmaxf(fv, 0.f) + 1e-10f);
        float l3 = log10f(s3 / (float)c3 + 1e-10f);
        float l5 = log10f(s5 / (float)c5 + 1e-10f);
        float f[8], zz8[8];
        f[0] = (l3 + 5.f) * (1.f / 3.f);
        f[1] = fminf(fmaxf(4.f * (l0 - l3), -4.f), 4.f);
        f[2] = fminf(fmaxf(4.f * (l5 - l3), -4.f), 4.f);
        f[3] = fv <= 0.f ? 1.f : 0.f;
        f[4] = pr[0] > 0.f ? log10f(pr[0]) + 2.f : -2.f;
        float musp = pr[1] * (1.f - pr[2]);
        f[5] = musp > 0.f ? log10f(musp) : -3.f;
        f[6] = (log_photons[n] - 5.5f) * 2.f;
        f[7] = 0.f;
        for (int e = 0; e < 8; ++e) zz8[e] = 0.f;
        store8(x0 + v * 16, f);
        store8(x0 + v * 16 + 8, zz8);
        xres[v] = l3;
    }
}

// AdamW on fp32 master weights (decoupled weight decay), gradient cleared after use.  Writes the
// bf16 weights and, for a convolution (taps > 0), the flipped transposed copy the data gradient
// runs on: wt[ci][taps-1-t][co] = w[co][t][ci].
__global__ void adamw_kernel(float* __restrict__ master, float* __restrict__ grad, float* __restrict__ m1,
                             float* __restrict__ m2, bf16* __restrict__ w16, bf16* __restrict__ wt16, long long n,
                             int cout, int taps, int cin, float lr, float b1, float b2, float eps, float wd,
                             float bc1, float bc2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float gr = grad[i];
        float a = b1 * m1[i] + (1.f - b1) * gr;
        float s = b2 * m2[i] + (1.f - b2) * gr * gr;
        m1[i] = a;
        m2[i] = s;
        float p = master[i];
        p -= lr * (wd * p + (a / bc1) / (sqrtf(s / bc2) + eps));
        master[i] = p;
        grad[i] = 0.f;
        bf16 pb = __float2bfloat16_rn(p);
        if (w16) w16[i] = pb;
        if (wt16 && taps > 0) {
            int ci = (int)(i % cin);
            int t = (int)((i / cin) % taps);
            int co = (int)(i / ((long long)cin * taps));
            wt16[((long long)ci * taps + (taps - 1 - t)) * cout + co] = pb;
        }
    }
}

thread_local char g_err[256];

int fail(const char* msg) {
    snprintf(g_err, sizeof(g_err), "%s", msg);
    return -1;
}

int launched() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "denoiser kernel launch: %s", cudaGetErrorString(e));
        return -(int)e;
    }
    return 0;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

int grid_for(long long work, int block) {
    long long g = (work + block - 1) / block;
    return (int)(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

template <int BM, int BN, int BK, int WARPS_M, int WARPS_N, int STAGES>
int conv_fwd_launch(const bf16* x, const bf16* w, const float* bias, const bf16* mask, bf16* y, Geo g, int cin,
                    int cout, int taps, int relu, cudaStream_t st) {
    constexpr int stage_bytes = (BM + BN) * BK * 2;
    constexpr int epi_bytes = BM * (BN + 8) * 2;
    constexpr int smem = STAGES * stage_bytes > epi_bytes ? STAGES * stage_bytes : epi_bytes;
    auto kern = conv_fwd_kernel<BM, BN, BK, WARPS_M, WARPS_N, STAGES>;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
    }
    dim3 grid((unsigned)((g.m + BM - 1) / BM), (unsigned)(cout / BN));
    kern<<<grid, 32 * WARPS_M * WARPS_N, smem, st>>>(x, w, bias, mask, y, g, cin, cout, taps, relu);
    return launched();
}

// Tile per output width: 128 voxels x (128 | 64 | 32 | 16) channels; narrow outputs take deeper
// K stages and fewer, taller warp tiles (two 16-row fragments per warp) so that each B fragment
// feeds more MMAs.
template <int BN>
int conv3_halo_launch(const bf16* x, const bf16* w, const float* bias, const bf16* mask, bf16* y, Geo g, int cin,
                      int cout, int relu, cudaStream_t st) {
    constexpr int smem_in = 400 * 32 + 27 * BN * 32;
    constexpr int smem_epi = 128 * (BN + 8) * 2;
    constexpr int smem = smem_in > smem_epi ? smem_in : smem_epi;
    auto kern = conv3_halo_kernel<BN>;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
    }
    const int tx = (g.w + 7) / 8, ty = (g.h + 7) / 8, tz = (g.d + 1) / 2;
    const long long tiles = (long long)g.nvol * tx * ty * tz;
    if (tiles >= (1LL << 31)) return fail("conv: too many tiles");
    kern<<<dim3((unsigned)tiles, (unsigned)(cout / BN)), 128, smem, st>>>(x, w, bias, mask, y, g, cin, cout, relu, tx, ty,
                                                                          tz);
    return launched();
}

// cuTensorMapEncodeTiled, found through the runtime (the engine links no driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    return fn;
}

template <int BN>
int conv3_tc_launch(const bf16* x, const bf16* w, const float* bias, const bf16* mask, bf16* y, Geo g, int cin,
                    int cout, int relu, cudaStream_t st) {
    using S = TcConvShape<BN>;
    if (!aligned16(x)) return fail("conv: the input must be 16-byte aligned");
    auto encode = tensor_map_encoder();
    if (!encode) return fail("conv: cuTensorMapEncodeTiled is not available");
    // activations [nvol][d][h][w][cin] as a 5-D tensor (channel fastest) with a 8 x 10 x 18 x 4 x 1 box
    CUtensorMap tmap;
    const cuuint64_t dims[5] = {(cuuint64_t)cin, (cuuint64_t)g.w, (cuuint64_t)g.h, (cuuint64_t)g.d, (cuuint64_t)g.nvol};
    const cuuint64_t strides[4] = {(cuuint64_t)cin * 2, (cuuint64_t)g.w * cin * 2, (cuuint64_t)g.h * g.w * cin * 2,
                                   (cuuint64_t)g.d * g.h * g.w * cin * 2};
    const cuuint32_t box[5] = {8, (cuuint32_t)S::HX, (cuuint32_t)S::HY, (cuuint32_t)S::HZ, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    if (encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16*>(x), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return fail("conv: cuTensorMapEncodeTiled rejected the activation layout");
    const int wbytes = (cin / 16) * S::WSLICE;
    const int limit = 227 * 1024;
    int stages = (limit - wbytes) / S::HALO;
    if (stages > S::MAX_STAGES) stages = S::MAX_STAGES;
    if (stages < 2) return fail("conv: weights of this layer do not fit in shared memory");
    // two CTAs per SM hide each other's waits better than a fourth halo stage does
    while (stages > 3 && 2 * (wbytes + stages * S::HALO + 2048) > 228 * 1024) --stages;
    const int smem = wbytes + stages * S::HALO;
    auto kern = conv3_tc_kernel<BN>;
    static int attr = 0;
    if (smem > attr) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = smem;
    }
    const int tx = (g.w + S::TX - 1) / S::TX, ty = (g.h + S::TY - 1) / S::TY;
    const long long tiles = (long long)g.nvol * ((g.d + S::TZ - 1) / S::TZ) * tx * ty;
    if (tiles >= (1LL << 31)) return fail("conv: too many tiles");
    // persistent CTAs: as many as shared memory lets stay resident on every SM
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = (228 * 1024) / (smem + 2048);
    if (per_sm > 8) per_sm = 8;
    if (per_sm < 1) per_sm = 1;
    const int ny = cout / BN;
    long long grid = (long long)sms * per_sm / ny;
    if (grid < 1) grid = 1;
    if (grid > tiles) grid = tiles;
    kern<<<dim3((unsigned)grid, (unsigned)ny), 192, smem, st>>>(tmap, w, bias, mask, y, g, cin, cout, relu, tx, ty,
                                                               (int)tiles, stages);
    return launched();
}

// Narrow 3x3x3 layers run on tcgen05 unless MCXG_DN_MMA_SYNC=1 selects the warp-level mma.sync
// halo kernel (kept as the measured baseline of the tensor-core port).
bool use_tcgen05() {
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("MCXG_DN_MMA_SYNC");
        v = (e && e[0] == '1') ? 0 : 1;
    }
    return v == 1;
}

int conv_fwd_dispatch(const bf16* x, const bf16* w, const float* bias, const bf16* mask, bf16* y, Geo g, int cin,
                      int cout, int taps, int relu, cudaStream_t st) {
    if (use_tcgen05() && taps == 27 && cin % 16 == 0) {
        if (cout % 32 == 0 && cout / 32 <= 3 && cout % 64 != 0)
            return conv3_tc_launch<32>(x, w, bias, mask, y, g, cin, cout, relu, st);
        if (cout % 32 != 0) return conv3_tc_launch<16>(x, w, bias, mask, y, g, cin, cout, relu, st);
    }
    // narrow 3x3x3 layers: halo tiles (each input voxel loaded once per tile, not once per tap)
    if (taps == 27 && cin % 16 == 0 && cout % 32 == 0 && cout / 32 <= 3 && cout % 64 != 0)
        return conv3_halo_launch<32>(x, w, bias, mask, y, g, cin, cout, relu, st);
    if (taps == 27 && cin % 16 == 0 && cout % 32 != 0)
        return conv3_halo_launch<16>(x, w, bias, mask, y, g, cin, cout, relu, st);
    if (cout % 128 == 0) return conv_fwd_launch<128, 128, 32, 2, 4, 4>(x, w, bias, mask, y, g, cin, cout, taps, relu, st);
    if (cout % 64 == 0) return conv_fwd_launch<128, 64, 32, 4, 2, 4>(x, w, bias, mask, y, g, cin, cout, taps, relu, st);
    if (cout % 32 == 0) return conv_fwd_launch<128, 32, 64, 4, 1, 3>(x, w, bias, mask, y, g, cin, cout, taps, relu, st);
    return conv_fwd_launch<128, 16, 64, 4, 1, 3>(x, w, bias, mask, y, g, cin, cout, taps, relu, st);
}

template <int BM>
int wgrad_launch(const bf16* dy, const bf16* x, float* dw, Geo g, int cin, int taps, cudaStream_t st) {
    constexpr int STAGES = 4;
    constexpr int smem = STAGES * (32 * BM + 32 * 64) * 2;
    auto kern = conv_wgrad_kernel<BM, STAGES>;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
    }
    const int ntiles = (taps * cin + 63) / 64;
    // about 4 CTAs per SM over the (column tile, voxel slice) grid, slices a multiple of 32 voxels
    long long want = 152 * 4 / ntiles;
    if (want < 1) want = 1;
    long long kslice = (g.m + want - 1) / want;
    kslice = ((kslice + 31) / 32) * 32;
    if (kslice < 256) kslice = 256;
    unsigned nsl = (unsigned)((g.m + kslice - 1) / kslice);
    kern<<<dim3((unsigned)ntiles, nsl), 128, smem, st>>>(dy, x, dw, g, cin, taps, kslice);
    return launched();
}

Geo make_geo(int nvol, int d, int h, int w) {
    Geo g;
    g.nvol = nvol;
    g.d = d;
    g.h = h;
    g.w = w;
    g.m = (long long)nvol * d * h * w;
    return g;
}

bool dims_ok(int nvol, int d, int h, int w) { return nvol > 0 && d > 0 && h > 0 && w > 0; }

}  // namespace

extern "C" {

const char* mcxg_dn_last_error(void) { return g_err; }

int mcxg_dn_check(void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "denoiser stream: %s", cudaGetErrorString(e));
        return -(int)e;
    }
    unsigned f = 0;
    e = cudaMemcpyFromSymbol(&f, g_dn_fault, sizeof(f));
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof(g_err), "denoiser fault word: %s", cudaGetErrorString(e));
        return -(int)e;
    }
    if (f) {
        const unsigned zero = 0;
        cudaMemcpyToSymbol(g_dn_fault, &zero, sizeof(zero));
        return fail("a tensor-core convolution gave up waiting for its MMAs (bounded wait); its output is invalid");
    }
    return 0;
}

int mcxg_dn_conv_fwd(const void* x, const void* w, const float* bias, const void* mask, void* y, int nvol, int d,
                     int h, int wd, int cin, int cout, int taps, int relu, void* stream) {
    if (!x || !w || !y || !dims_ok(nvol, d, h, wd)) return fail("conv: null tensor or empty volume");
    if (cin % 8 || cout % 16 || cin <= 0 || cout <= 0) return fail("conv: cin must be a multiple of 8, cout of 16");
    if (taps != 1 && taps != 27) return fail("conv: taps must be 1 or 27");
    if (!aligned16(x) || !aligned16(w) || !aligned16(y) || (mask && !aligned16(mask)))
        return fail("conv: tensors must be 16-byte aligned");
    Geo g = make_geo(nvol, d, h, wd);
    if (g.m >= (1LL << 31) || d >= 1024 || h >= 1024 || wd >= 1024) return fail("conv: volume too large");
    return conv_fwd_dispatch(static_cast<const bf16*>(x), static_cast<const bf16*>(w), bias,
                             static_cast<const bf16*>(mask), static_cast<bf16*>(y), g, cin, cout, taps, relu,
                             static_cast<cudaStream_t>(stream));
}

int mcxg_dn_conv_wgrad(const void* dy, const void* x, float* dw, int nvol, int d, int h, int wd, int cin, int cout,
                       int taps, void* stream) {
    if (!dy || !x || !dw || !dims_ok(nvol, d, h, wd)) return fail("wgrad: null tensor or empty volume");
    if (cin % 16 || cin <= 0) return fail("wgrad: input channels must be a multiple of 16");
    if (taps != 1 && taps != 27) return fail("wgrad: taps must be 1 or 27");
    if (!aligned16(dy) || !aligned16(x)) return fail("wgrad: tensors must be 16-byte aligned");
    Geo g = make_geo(nvol, d, h, wd);
    auto st = static_cast<cudaStream_t>(stream);
    auto DY = static_cast<const bf16*>(dy);
    auto X = static_cast<const bf16*>(x);
    switch (cout) {
        case 16: return wgrad_launch<16>(DY, X, dw, g, cin, taps, st);
        case 32: return wgrad_launch<32>(DY, X, dw, g, cin, taps, st);
        case 64: return wgrad_launch<64>(DY, X, dw, g, cin, taps, st);
        case 128: return wgrad_launch<128>(DY, X, dw, g, cin, taps, st);
        default: return fail("wgrad: output channels must be 16, 32, 64 or 128");
    }
}

int mcxg_dn_bias_grad(const void* dy, float* db, long long m, int c, void* stream) {
    if (!dy || !db || m <= 0) return fail("bias grad: null tensor or no voxels");
    if (c <= 0 || 256 % c) return fail("bias grad: channels must divide 256");
    long long rows = 4096;
    unsigned blocks = (unsigned)((m + rows - 1) / rows);
    bias_grad_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(dy), db, m, c, rows);
    return launched();
}

int mcxg_dn_pool(const void* x, void* y, int nvol, int d, int h, int w, int c, void* stream) {
    if (!x || !y || !dims_ok(nvol, d, h, w) || (d | h | w) & 1 || c % 8) return fail("pool: bad shape");
    long long work = (long long)nvol * (d / 2) * (h / 2) * (w / 2) * (c / 8);
    pool_kernel<<<grid_for(work, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(x), static_cast<bf16*>(y), nvol, d, h, w, c);
    return launched();
}

int mcxg_dn_upcat(const void* low, const void* skip, void* cat, int nvol, int d, int h, int w, int c1, int c2,
                  void* stream) {
    if (!low || !skip || !cat || !dims_ok(nvol, d, h, w) || (d | h | w) & 1 || c1 % 8 || c2 % 8)
        return fail("upcat: bad shape");
    long long work = (long long)nvol * d * h * w * ((c1 + c2) / 8);
    upcat_kernel<<<grid_for(work, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(low), static_cast<const bf16*>(skip), static_cast<bf16*>(cat), nvol, d, h, w, c1, c2);
    return launched();
}

int mcxg_dn_upcat_bwd(const void* dcat, const void* low, void* dlow, int nvol, int d, int h, int w, int c1, int c2,
                      void* stream) {
    if (!dcat || !low || !dlow || !dims_ok(nvol, d, h, w) || (d | h | w) & 1 || c1 % 8 || c2 % 8)
        return fail("upcat backward: bad shape");
    long long work = (long long)nvol * (d / 2) * (h / 2) * (w / 2) * (c1 / 8);
    upcat_bwd_kernel<<<grid_for(work, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(dcat), static_cast<const bf16*>(low), static_cast<bf16*>(dlow), nvol, d, h, w, c1, c2);
    return launched();
}

int mcxg_dn_unpool_add(const void* dpool, const void* dcat, const void* enc, void* denc, int nvol, int d, int h, int w,
                       int c1, int c, void* stream) {
    if (!dpool || !enc || !denc || !dims_ok(nvol, d, h, w) || (d | h | w) & 1 || c % 8 || c1 % 8)
        return fail("unpool: bad shape");
    long long work = (long long)nvol * d * h * w * (c / 8);
    unpool_add_kernel<<<grid_for(work, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(dpool), static_cast<const bf16*>(dcat), static_cast<const bf16*>(enc),
        static_cast<bf16*>(denc), nvol, d, h, w, c1, c);
    return launched();
}

int mcxg_dn_head(const void* act, const float* xres, const float* w, const float* b, const float* target,
                 const float* valid, float* out, void* dact, float* dw, float* db, float* loss, long long m, float inv,
                 void* stream) {
    if (!act || !xres || !w || !b || m <= 0) return fail("head: null tensor or no voxels");
    if (target && (!valid || !dact || !dw || !db || !loss)) return fail("head: training needs valid/dact/dw/db/loss");
    if (!target && !out) return fail("head: nothing to write");
    head_kernel<<<grid_for(m, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(act), xres, w, b, target, valid, out, static_cast<bf16*>(dact), dw, db, loss, m, inv);
    return launched();
}

int mcxg_dn_pack(const float* flux, const uint8_t* label, const float* props, const float* log_photons, void* x0,
                 float* xres, int nvol, int d, int h, int w, int nprop, void* stream) {
    if (!flux || !label || !props || !log_photons || !x0 || !xres || !dims_ok(nvol, d, h, w) || nprop <= 0)
        return fail("pack: bad arguments");
    Geo g = make_geo(nvol, d, h, w);
    pack_kernel<<<grid_for(g.m, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        flux, label, props, log_photons, static_cast<bf16*>(x0), xres, g, nprop);
    return launched();
}

int mcxg_dn_adamw(float* master, float* grad, float* m1, float* m2, void* w16, void* wt16, long long n, int cout,
                  int taps, int cin, float lr, float b1, float b2, float eps, float wd, int step, void* stream) {
    if (!master || !grad || !m1 || !m2 || n <= 0 || step < 1) return fail("adamw: bad arguments");
    if (wt16 && (taps <= 0 || (long long)cout * taps * cin != n)) return fail("adamw: transposed copy needs the shape");
    float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
    adamw_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        master, grad, m1, m2, static_cast<bf16*>(w16), static_cast<bf16*>(wt16), n, cout, taps, cin, lr, b1, b2, eps,
        wd, bc1, bc2);
    return launched();
}

}  // extern "C"
