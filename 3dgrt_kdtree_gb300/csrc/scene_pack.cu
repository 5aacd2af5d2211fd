// scene_pack.cu -- scene ingest on the device.
//
// Every scene upload goes through here: the caller's 64-float Gaussian
// records (the reference's Gaussian struct, Kd-treeConverter.h:319-335) are
// either copied to the device as they are (kdgr_scene_create) or already
// there (kdgr_scene_create_device, kdgr_read_ply_device), and these kernels
// write the per-Gaussian arrays each render form reads -- one thread per
// Gaussian, straight into the scene's SoA arrays:
//   * inverse scales as the reference's caller leaves them (the FP32 1/s of
//     Kd-treeConverterMain.cpp:3636-3650 unless the records are inverted);
//   * SH coefficients coefficient-major (f_dc, then f_rest channel-major
//     re-ordered, cudaRenderer.cu:494-499);
//   * the plain kernel's 64-byte test record: position, opacity, inverse
//     scale, its IEEE reciprocal (cudaRenderer.cu:1091) and the quaternion;
//   * the fast form's rows of M = diag(1/s) R^T and b = M mu, computed in
//     FP64 from R^T of quaternionWXYZToMatrixTranspose (cudaRenderer.cu:
//     808-828) and stored FP32; the opacity array;
//   * the precision form's staging words (FP32 mean, FP16 entries of M), BF16
//     SH and the flag of Gaussians whose scale ratio exceeds 1e3 (or whose
//     factors leave the FP16 range).
// The unit is built with --fmad=false and IEEE division and square root, and
// the double-precision steps are spelled as __d*_rn intrinsics, so every
// value equals the host computation of the same formula bit for bit.
//
// PLY activation (loadGaussiansFromPly, Kd-treeConverterMain.cpp:1652-1769):
// the vertex block is streamed to the device in chunks through two pinned
// buffers and activated by k_ply_activate while the next chunk is read.  exp,
// log and pow are evaluated in double and rounded once to float, as the host
// loader does; CUDA's double functions are within 1 ulp of double, so the
// float results equal the correctly rounded ones except in cases of
// vanishing probability (a double result within 2^-52 of a float rounding
// boundary).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "scene.h"

namespace kdgr {
namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// R^T of quaternionWXYZToMatrixTranspose (cudaRenderer.cu:808-828) in double
// from the FP32 quaternion (w, x, y, z).
__device__ __forceinline__ void quat_rt_d(const float* q, double m[3][3]) {
  const double r = q[0], x = q[1], y = q[2], z = q[3];
  const double xx = dm(x, x), yy = dm(y, y), zz = dm(z, z), xy = dm(x, y), xz = dm(x, z), yz = dm(y, z);
  const double rx = dm(r, x), ry = dm(r, y), rz = dm(r, z);
  m[0][0] = ds(1.0, dm(2.0, da(yy, zz)));
  m[0][1] = dm(2.0, da(xy, rz));
  m[0][2] = dm(2.0, ds(xz, ry));
  m[1][0] = dm(2.0, ds(xy, rz));
  m[1][1] = ds(1.0, dm(2.0, da(xx, zz)));
  m[1][2] = dm(2.0, da(yz, rx));
  m[2][0] = dm(2.0, da(xz, ry));
  m[2][1] = dm(2.0, ds(yz, rx));
  m[2][2] = ds(1.0, dm(2.0, da(xx, yy)));
}

__global__ void k_pack(const float* __restrict__ rec, uint32_t n, int inverted, PackOut o) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float r[64];
  const float4* src = reinterpret_cast<const float4*>(rec) + 16ull * i;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const float4 v = __ldg(src + k);
    r[4 * k] = v.x;
    r[4 * k + 1] = v.y;
    r[4 * k + 2] = v.z;
    r[4 * k + 3] = v.w;
  }
  float gs[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) gs[c] = inverted ? r[4 + c] : __fdiv_rn(1.0f, r[4 + c]);
  float sh[48];
#pragma unroll
  for (int c = 0; c < 3; ++c) sh[c] = r[12 + c];
#pragma unroll
  for (int k = 1; k < 16; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) sh[3 * k + c] = r[15 + 15 * c + (k - 1)];
  if (o.sh) {
    float4* d = o.sh + 12ull * i;
#pragma unroll
    for (int k = 0; k < 12; ++k) d[k] = make_float4(sh[4 * k], sh[4 * k + 1], sh[4 * k + 2], sh[4 * k + 3]);
  }
  if (o.giscl) {
#pragma unroll
    for (int c = 0; c < 3; ++c) o.giscl[3ull * i + c] = gs[c];
  }
  if (o.test) {  // particleScale = 1 / giscl, cudaRenderer.cu:1091
    float4* d = o.test + 4ull * i;
    d[0] = make_float4(r[0], r[1], r[2], r[3]);
    d[1] = make_float4(gs[0], gs[1], gs[2], __fdiv_rn(1.0f, gs[0]));
    d[2] = make_float4(__fdiv_rn(1.0f, gs[1]), __fdiv_rn(1.0f, gs[2]), r[8], r[9]);
    d[3] = make_float4(r[10], r[11], 0.f, 0.f);
  }
  if (o.opacity) o.opacity[i] = r[3];
  double m[3][3];
  quat_rt_d(r + 8, m);
  if (o.fast) {  // rows of M = diag(1/s) R^T and b = M mu, FP64 -> FP32
    float4* d = o.fast + 3ull * i;
#pragma unroll
    for (int row = 0; row < 3; ++row) {
      const double sc = gs[row];
      double b = 0.0;
      float t[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double mv = dm(sc, m[row][c]);
        t[c] = (float)mv;
        b = da(b, dm(mv, (double)r[c]));
      }
      d[row] = make_float4(t[0], t[1], t[2], (float)b);
    }
  }
  if (o.packed) {
    // M in FP64 -> FP32 -> FP16; FP32 mean; flagged when the scale ratio
    // exceeds kAnisoRatio or an entry leaves the FP16 range
    const double smax = __drcp_rn(fmin(fmin((double)gs[0], (double)gs[1]), (double)gs[2]));
    const double smin = __drcp_rn(fmax(fmax((double)gs[0], (double)gs[1]), (double)gs[2]));
    float mf[3][3];
    double mmax = 0.0;
#pragma unroll
    for (int row = 0; row < 3; ++row)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double v = dm((double)gs[row], m[row][c]);
        mf[row][c] = (float)v;
        mmax = fmax(mmax, fabs(v));
      }
    auto pk = [](float a, float b) {
      const __half2 h = __floats2half2_rn(a, b);
      uint32_t w;
      memcpy(&w, &h, 4);
      return w;
    };
    uint32_t* p = o.packed + 8ull * i;
    p[0] = __float_as_uint(r[0]);
    p[1] = __float_as_uint(r[1]);
    p[2] = __float_as_uint(r[2]);
    p[3] = pk(mf[2][2], 0.f);
    p[4] = pk(mf[0][0], mf[0][1]);
    p[5] = pk(mf[0][2], mf[1][0]);
    p[6] = pk(mf[1][1], mf[1][2]);
    p[7] = pk(mf[2][0], mf[2][1]);
    o.aniso[i] = (smax > dm(kAnisoRatio, smin) || mmax > 30000.0) ? 1 : 0;
  }
  if (o.sh_bf16) {
    uint32_t* d = reinterpret_cast<uint32_t*>(o.sh_bf16 + 6ull * i);
#pragma unroll
    for (int k = 0; k < 24; ++k) {
      const __nv_bfloat16 lo = __float2bfloat16_rn(sh[2 * k]), hi = __float2bfloat16_rn(sh[2 * k + 1]);
      uint16_t a, b;
      memcpy(&a, &lo, 2);
      memcpy(&b, &hi, 2);
      d[k] = (uint32_t)a | ((uint32_t)b << 16);
    }
  }
}

// Source fields of the FP64 precompute for flagged Gaussian i (table entry
// aidx[i]): inverse scale x3, quaternion w,x,y,z, mean x3.
__global__ void k_gather_aniso(const float* __restrict__ rec, const float* __restrict__ giscl,
                               const uint32_t* __restrict__ aidx, uint32_t n, float* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t a = aidx[i];
  if (a == 0xFFFFFFFFu) return;
  const float* r = rec + 64ull * i;
  float* d = out + 10ull * a;
  d[0] = giscl[3ull * i];
  d[1] = giscl[3ull * i + 1];
  d[2] = giscl[3ull * i + 2];
  for (int k = 0; k < 4; ++k) d[3 + k] = r[8 + k];
  for (int k = 0; k < 3; ++k) d[7 + k] = r[k];
}

// ------------------------------------------------------------------ PLY
__device__ __forceinline__ float ld_f32(const uint8_t* p) {
  float x;
  memcpy(&x, p, 4);  // vertex fields need not be 4-byte aligned
  return x;
}

__device__ __forceinline__ float exp_f(float x) { return (float)exp((double)x); }

// calcKernelScale (Gaussian.h:6-15), ADAPTIVE_KERNEL_CLAMPING, KERNEL_DEGREE 4.
__device__ __forceinline__ float kernel_scale(float density) {
  const float min_resp = fminf(__fdiv_rn(0.0113f, density), 0.97f);
  const float a = -4.5f / 81.0f;
  const float l = (float)log((double)min_resp);
  return (float)pow((double)__fdiv_rn(l, a), 0.25);
}

// One thread per vertex of the chunk: the activation of loadGaussiansFromPly
// (Kd-treeConverterMain.cpp:1727-1747) into the vertex's 64-float record.
__global__ void k_ply_activate(const uint8_t* __restrict__ raw, uint32_t n, uint32_t stride, PlyLayout lay,
                               float* __restrict__ rec) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint8_t* v = raw + (size_t)i * stride;
  float r[64];
#pragma unroll
  for (int k = 0; k < 64; ++k) r[k] = 0.f;
  r[0] = ld_f32(v + lay.off[0]);
  r[1] = ld_f32(v + lay.off[1]);
  r[2] = ld_f32(v + lay.off[2]);
  const float op = __fdiv_rn(1.0f, __fadd_rn(1.0f, exp_f(-ld_f32(v + lay.off[3]))));  // sigmoid, :1729
  r[3] = op;
#pragma unroll
  for (int c = 0; c < 3; ++c) r[4 + c] = exp_f(ld_f32(v + lay.off[4 + c]));  // :1731-1734
  float q[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) q[c] = ld_f32(v + lay.off[7 + c]);
  // fMyVecNormalize4D (:1568-1577)
  const float len_sq =
      __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(q[0], q[0]), __fmul_rn(q[1], q[1])), __fmul_rn(q[2], q[2])),
                __fmul_rn(q[3], q[3]));
  if (len_sq > 0.00001f) {
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(len_sq));
#pragma unroll
    for (int c = 0; c < 4; ++c) q[c] = __fmul_rn(q[c], inv);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) r[8 + c] = q[c];
  r[7] = kernel_scale(op);
#pragma unroll
  for (int c = 0; c < 3; ++c) r[12 + c] = ld_f32(v + lay.off[11 + c]);
  if (lay.off[14] >= 0)
    for (int k = 0; k < 45; ++k) r[15 + k] = ld_f32(v + lay.off[14] + 4 * k);
  float4* d = reinterpret_cast<float4*>(rec) + 16ull * i;
#pragma unroll
  for (int k = 0; k < 16; ++k) d[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
}

}  // namespace

cudaError_t launch_pack(const float* d_rec, uint32_t n, bool inverted, const PackOut& out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_pack<<<(n + 127) / 128, 128, 0, st>>>(d_rec, n, inverted ? 1 : 0, out);
  return cudaGetLastError();
}

cudaError_t launch_gather_aniso(const float* d_rec, const float* d_giscl, const uint32_t* d_aidx, uint32_t n,
                                float* d_out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_gather_aniso<<<(n + 255) / 256, 256, 0, st>>>(d_rec, d_giscl, d_aidx, n, d_out);
  return cudaGetLastError();
}

cudaError_t launch_ply_activate(const uint8_t* d_raw, uint32_t n, uint32_t stride, const PlyLayout& lay,
                                float* d_rec, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_ply_activate<<<(n + 127) / 128, 128, 0, st>>>(d_raw, n, stride, lay, d_rec);
  return cudaGetLastError();
}

}  // namespace kdgr
