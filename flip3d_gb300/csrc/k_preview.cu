/*
 * k_preview.cu — the reference's point-splat preview (write_frame,
 * src/flip3D.cpp:1133-1192) into a headless device buffer, and its BMP
 * writer (write_bmp, src/write_bmp.cpp).
 *
 * Every liquid particle is rotated (buildRotationMatrix(-0.2, 0.2),
 * transform), projected, and blends the same colour into the 2x2 pixels
 * below and left of its projection: image = a*c + (1 - a)*image per
 * channel, with a = exp(-DENSITY*N/23). The same affine map applied k times
 * gives the same floats whatever the order of the particles, so a pixel's
 * value depends only on how many particles cover it: the first kernel
 * counts the covers with integer atomics (deterministic), the second
 * applies the reference's blend expression that many times from black and
 * converts to bytes as the reference does. The projection reproduces the
 * reference's float/double mix (nvcc -fmad=false).
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "devcommon.cuh"

namespace {

constexpr int PBLK = 256;

struct PreviewConst {
  int width, height, np;
  float R[3][3];
  float a;          /* blueColor[3] */
  float col[3];     /* blueColor[0..2] */
  float winrate;
};

__global__ void k_preview_count(PreviewConst c, const float *__restrict__ px,
                                const float *__restrict__ py, const float *__restrict__ pz,
                                const uint8_t *__restrict__ type, uint32_t *__restrict__ cnt) {
  const int q = blockIdx.x * PBLK + threadIdx.x;
  if (q >= c.np || type[q] != CELL_FLUID) return;
  const float eye = 2.0f, offset = 0.3f;
  float p0[3] = {(float)((double)px[q] - 0.5), (float)((double)py[q] - 0.5),
                 (float)((double)pz[q] - 0.5)};
  float p[3];
  for (int i = 0; i < 3; i++) {
    p[i] = 0.0f;
    for (int k = 0; k < 3; k++) p[i] += c.R[i][k] * p0[k];
  }
  const float z = (float)((double)offset + 0.5 + (double)p[2]);
  const float x = (float)((double)(eye / (eye + z)) * ((double)p[0] + 0.05));
  const float y = (float)((double)(eye / (eye + z)) * ((double)p[1] + 0.25));
  const double hw = (double)c.winrate / 2.0;
  if (!((double)x > -0.5 && (double)x < 0.5 && (double)y > -hw && (double)y < hw)) return;
  const int i = (int)((double)c.width * ((double)x + 0.5));
  const int j = (int)((double)c.width * ((double)y + hw));
  for (int ni = i - 1; ni < i + 1; ni++)
    for (int nj = j - 1; nj < j + 1; nj++)
      if (ni > 0 && ni < c.width && nj > 0 && nj < c.height)
        atomicAdd(cnt + (size_t)ni + (size_t)nj * c.width, 1u);
}

/* image = a*c + (1.0 - a)*image, k times from 0; bytes = 255*min(1, image) */
__global__ void k_preview_resolve(PreviewConst c, const uint32_t *__restrict__ cnt,
                                  uint8_t *__restrict__ rgba) {
  const size_t pix = (size_t)blockIdx.x * PBLK + threadIdx.x;
  if (pix >= (size_t)c.width * c.height) return;
  const uint32_t k = cnt[pix];
  const double keep = 1.0 - (double)c.a;
  for (int ch = 0; ch < 3; ch++) {
    const double ac = (double)(c.a * c.col[ch]);
    float v = 0.0f;
    for (uint32_t t = 0; t < k; t++) {
      const float nv = (float)(ac + keep * (double)v);
      if (nv == v) break; /* a fixed point: every further blend returns it */
      v = nv;
    }
    rgba[4 * pix + ch] = (uint8_t)(255.0 * fmin(1.0, (double)v));
  }
  rgba[4 * pix + 3] = (uint8_t)(255.0 * fmin(1.0, 1.0));
}

/* buildRotationMatrix (src/flip3D.cpp:1105-1121) in the reference's FLOAT */
void rotation(float xrad, float yrad, float R[3][3]) {
  const float Rx[3][3] = {{1, 0, 0},
                          {0, (float)cos((double)xrad), (float)-sin((double)xrad)},
                          {0, (float)sin((double)xrad), (float)cos((double)xrad)}};
  const float Ry[3][3] = {{(float)cos((double)yrad), 0, (float)sin((double)yrad)},
                          {0, 1, 0},
                          {(float)-sin((double)yrad), 0, (float)cos((double)yrad)}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      R[i][j] = 0.0f;
      for (int k = 0; k < 3; k++) R[i][j] += Rx[i][k] * Ry[k][j];
    }
}

} // namespace

extern "C" {

int flipgpu_preview(FlipGpu *h, uint8_t *rgba, int width, int height, int on_device) {
  if (!h || !rgba || width < 2 || height < 2) return FLIPGPU_EINVAL;
  PreviewConst c;
  std::memset(&c, 0, sizeof c);
  c.width = width;
  c.height = height;
  c.np = h->np;
  rotation(-0.2f, 0.2f, c.R);
  const float blue[4] = {0.3f, 0.5f, 0.8f,
                         (float)exp(-(double)h->prm.density * h->n / 23.0)};
  c.col[0] = blue[0];
  c.col[1] = blue[1];
  c.col[2] = blue[2];
  c.a = blue[3];
  c.winrate = (float)height / (float)width;
  const size_t npix = (size_t)width * height;
  uint32_t *cnt = nullptr;
  uint8_t *dbuf = nullptr;
  cudaError_t e = cudaMalloc(&cnt, npix * sizeof(uint32_t));
  if (e == cudaSuccess && !on_device) e = cudaMalloc(&dbuf, 4 * npix);
  if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, npix * sizeof(uint32_t), h->stream);
  if (e == cudaSuccess && h->np > 0) {
    k_preview_count<<<(h->np + PBLK - 1) / PBLK, PBLK, 0, h->stream>>>(c, h->px, h->py, h->pz,
                                                                        h->type, cnt);
    e = cudaGetLastError();
  }
  uint8_t *out = on_device ? rgba : dbuf;
  if (e == cudaSuccess) {
    k_preview_resolve<<<(unsigned)((npix + PBLK - 1) / PBLK), PBLK, 0, h->stream>>>(c, cnt, out);
    e = cudaGetLastError();
  }
  FG_LAUNCHED(h, h->np > 0 ? 2 : 1);
  if (e == cudaSuccess && !on_device)
    e = cudaMemcpyAsync(rgba, dbuf, 4 * npix, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(cnt);
  if (dbuf) cudaFree(dbuf);
  if (e != cudaSuccess) {
    snprintf(h->err, sizeof h->err, "preview: %s", cudaGetErrorString(e));
    return FLIPGPU_ECUDA;
  }
  return FLIPGPU_OK;
}

/* write_bmp (src/write_bmp.cpp): 54-byte header, 24-bit BGR rows of
 * (3*(width+1)/4)*4 bytes, rows in buffer order */
int flipgpu_write_bmp(const char *path, const uint8_t *rgba, int width, int height) {
  if (!path || !rgba || width < 1 || height < 1) return FLIPGPU_EINVAL;
  const int bpl = (3 * (width + 1) / 4) * 4;
  std::vector<uint8_t> out(54 + (size_t)bpl * height, 0);
  auto put32 = [&](size_t at, uint32_t v) {
    for (int b = 0; b < 4; b++) out[at + b] = (uint8_t)(v >> (8 * b));
  };
  auto put16 = [&](size_t at, uint16_t v) {
    out[at] = (uint8_t)v;
    out[at + 1] = (uint8_t)(v >> 8);
  };
  out[0] = 'B';
  out[1] = 'M';
  put32(2, (uint32_t)(54 + bpl * height));
  put32(6, 0);
  put32(10, 54);
  put32(14, 40);
  put32(18, (uint32_t)width);
  put32(22, (uint32_t)height);
  put16(26, 1);
  put16(28, 24);
  put32(30, 0);
  put32(34, (uint32_t)(bpl * height));
  for (int v = 0; v < height; v++)
    for (int j = 0; j < width; j++) {
      const size_t pos = 4 * ((size_t)width * v + j), o = 54 + (size_t)v * bpl + 3 * (size_t)j;
      out[o] = rgba[pos + 2];
      out[o + 1] = rgba[pos + 1];
      out[o + 2] = rgba[pos];
    }
  FILE *fp = fopen(path, "wb");
  if (!fp) return FLIPGPU_EINVAL;
  const bool ok = fwrite(out.data(), 1, out.size(), fp) == out.size();
  return (fclose(fp) == 0 && ok) ? FLIPGPU_OK : FLIPGPU_EINVAL;
}

} // extern "C"
