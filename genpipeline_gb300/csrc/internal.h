// internal.h -- functions shared between the translation units of libgbsimp.
#pragma once

#include "common.cuh"

namespace gbs {
int apply_f32(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
              const float *p, float *y, const uint8_t *mask, cudaStream_t st);
int apply_f64(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
              const double *p, double *y, const uint8_t *mask, cudaStream_t st);
int filter_launch(const gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, int mode, const float *hs,
                  const float *in, const uint8_t *preserved, float *out, cudaStream_t st);
// A 4 KiB pinned host buffer private to the calling thread (for small status reads).
void *thread_pinned();
}  // namespace gbs
