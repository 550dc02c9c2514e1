/*
 * conv_tc.h — the U-Net's forward 3x3x3 convolution on the tcgen05 tensor
 * cores (k_conv_tc.cu). Activations are BF16 [sample][cell][channel] with
 * cells x-major; weights come packed by conv_tc_pack.
 */
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

/* whether conv_tc_launch handles this level size and channel counts */
bool conv_tc_supported(int n, int cin, int cout);

/* W[tap][ci][co] (FP32, tap = (di*3 + dj)*3 + dk) into the operand layout
 * of conv_tc_launch; out holds 27*cin*cout BF16 */
cudaError_t conv_tc_pack(cudaStream_t st, int cin, int cout, const float *W, __nv_bfloat16 *out);

/* Y = (relu)(conv3x3x3(X, W) + bias) over batch samples of an n^3 grid
 * (bias may be null). An expired bounded wait inside the kernel sets *err
 * to 1; the launch itself reports configuration errors. */
cudaError_t conv_tc_launch(cudaStream_t st, int n, int batch, int cin, int cout,
                           const __nv_bfloat16 *X, const __nv_bfloat16 *Wtc, const float *bias,
                           __nv_bfloat16 *Y, int relu, int *err);

/* one-time per-device setup (shared-memory limits); 0 on success */
int conv_tc_init_device();
