/* C ABI of the fluence denoiser's GPU kernels (libmcx_gb300.so).
 *
 * The reference MCX has no learned denoiser (its optional ANLM filter is a separate, non-learned
 * submodule); these entry points serve the engine's own MC + denoiser pipeline
 * (mcx_gb300/denoise.py): a 4-level 3D U-Net trained on low-/high-photon fluence pairs that this
 * engine simulates.  All pointers are device pointers; `stream` is a cudaStream_t (NULL = legacy
 * default stream).  Activations are bf16, channels-last [nvol][d][h][w][c]; convolution weights
 * bf16 [cout][taps][cin] with tap = dz*9 + dy*3 + dx; gradients, master weights and Adam moments
 * fp32.  Every call returns 0 on success, -1 for invalid arguments, or -(cudaError) for a launch
 * failure; mcxg_dn_last_error() describes the last failure of the calling thread.
 */
#ifndef MCXG_DENOISE_H
#define MCXG_DENOISE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

const char* mcxg_dn_last_error(void);

/* Waits for `stream` and reports whether a tensor-core convolution launched before gave up a
 * bounded wait for its MMAs (then its output is invalid): 0, or -1 with a message. */
int mcxg_dn_check(void* stream);

/* y = act(conv3d(x, w) + bias) [* (mask > 0)]: 3x3x3 (taps = 27, zero padding 1) or 1x1x1
 * (taps = 1) convolution, stride 1.  cin, cout multiples of 16.  bias and mask may be NULL;
 * relu != 0 applies max(0, .) before the mask.  Run on the transposed weights the optimiser
 * writes (mcxg_dn_adamw), the same call is the data gradient, with the layer input as mask. */
int mcxg_dn_conv_fwd(const void* x, const void* w, const float* bias, const void* mask, void* y, int nvol, int d,
                     int h, int w_, int cin, int cout, int taps, int relu, void* stream);

/* dw[cout][taps][cin] += sum over voxels of dy[v][co] * x[v + off(tap)][ci] (fp32 atomics).
 * cout in {16, 32, 64, 128}; cin a multiple of 16. */
int mcxg_dn_conv_wgrad(const void* dy, const void* x, float* dw, int nvol, int d, int h, int w_, int cin, int cout,
                       int taps, void* stream);

/* db[c] += sum over m voxels of dy[v][c]; c divides 256. */
int mcxg_dn_bias_grad(const void* dy, float* db, long long m, int c, void* stream);

/* 2x2x2 average pooling of x [nvol][d][h][w][c] (even d, h, w) into y [nvol][d/2][h/2][w/2][c]. */
int mcxg_dn_pool(const void* x, void* y, int nvol, int d, int h, int w, int c, void* stream);

/* cat[v] = (low[parent(v)] (c1 channels), skip[v] (c2 channels)); (d, h, w) is the fine grid. */
int mcxg_dn_upcat(const void* low, const void* skip, void* cat, int nvol, int d, int h, int w, int c1, int c2,
                  void* stream);

/* dlow[u][c] = sum over u's 8 children of dcat[child][c] (c < c1), times (low[u][c] > 0). */
int mcxg_dn_upcat_bwd(const void* dcat, const void* low, void* dlow, int nvol, int d, int h, int w, int c1, int c2,
                      void* stream);

/* denc[v][c] = (dpool[parent(v)][c] / 8 + dcat[v][c1 + c]) * (enc[v][c] > 0); dcat may be NULL. */
int mcxg_dn_unpool_add(const void* dpool, const void* dcat, const void* enc, void* denc, int nvol, int d, int h, int w,
                       int c1, int c, void* stream);

/* Head over m voxels: out[v] = xres[v] + b[0] + sum_c w[c] * act[v][c] (16 channels).  With a
 * target: loss += sum |out - target| * valid; with g = sign(out - target) * valid * inv,
 * dact[v][c] = g * w[c] * (act[v][c] > 0), dw[c] += g * act[v][c], db[0] += g.  out may be NULL
 * when training. */
int mcxg_dn_head(const void* act, const float* xres, const float* w, const float* b, const float* target,
                 const float* valid, float* out, void* dact, float* dw, float* db, float* loss, long long m, float inv,
                 void* stream);

/* Input features of nvol volumes of d x h x w voxels: fluence (fp32, normalised as MCX writes
 * it, x fastest), labels (uint8) with per-volume media tables props[nvol][nprop][4] (mua, mus, g,
 * n), and log10(photons) per volume -> x0 (bf16, 16 channels: with l0, l3, l5 the log10 of the
 * fluence and of its 3x3x3 and 5x5x5 in-bounds means, the scaled l3, 4 (l0 - l3), 4 (l5 - l3),
 * an empty-voxel flag, log10 mua, log10 reduced scattering, a photon-count code) and xres = l3. */
int mcxg_dn_pack(const float* flux, const uint8_t* label, const float* props, const float* log_photons, void* x0,
                 float* xres, int nvol, int d, int h, int w, int nprop, void* stream);

/* One AdamW step (decoupled weight decay) over n fp32 parameters; clears grad.  Writes bf16
 * weights to w16 (may be NULL) and, for a convolution, the flipped transposed copy
 * wt16[ci][taps-1-t][co] (NULL to skip; needs cout * taps * cin == n).  step counts from 1. */
int mcxg_dn_adamw(float* master, float* grad, float* m1, float* m2, void* w16, void* wt16, long long n, int cout,
                  int taps, int cin, float lr, float b1, float b2, float eps, float wd, int step, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MCXG_DENOISE_H */
