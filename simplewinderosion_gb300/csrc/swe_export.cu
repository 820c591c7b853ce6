// Observables the reference's app loop reads after each erode call, built on
// the device:
//   the wind map, one RGBA texel per cell,
//     (0.5(1+erf(2 momentumx)), 0.5(1+erf(2 momentumy)), 0.5(1+erf(2 momentumz)), 1)
//     (SimpleWindErosion.cpp:224-230; erf of a float argument there is the
//     float erf overload);
//   the surface vertices updatenode writes for rendering (cellpool.h:302-333):
//     per cell the position P = (x, mapscale h, z), the normal quad::_normal,
//     and the edges T - P, B - P to the +x and +z neighbours (heights off the
//     map read 0, node::height, cellpool.h:256-260). This file is compiled
//     with -fmad=false, so the float operations are the reference's.
#include <cuda_runtime.h>

#include "swe_device.cuh"
#include "swe_kernels.h"

namespace swe {
namespace {

__global__ void k_windmap(const float* __restrict__ mx, const float* __restrict__ my, const float* __restrict__ mz,
                          long n, float4* __restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float4 t;
    t.x = 0.5f * (1.0f + erff(2.0f * mx[i]));
    t.y = 0.5f * (1.0f + erff(2.0f * my[i]));
    t.z = 0.5f * (1.0f + erff(2.0f * mz[i]));
    t.w = 1.0f;
    out[i] = t;
  }
}

__global__ void k_vertices(const float* __restrict__ H, Consts c, float* __restrict__ out) {
  const long n = (long)c.nx * c.nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i / c.nz), z = (int)(i % c.nz);
    auto h = [&](int a, int b) { return (a < 0 || b < 0 || a >= c.nx || b >= c.nz) ? 0.0f : H[(long)a * c.nz + b]; };
    const float py = c.mapscale * h(x, z);
    const V3 nv = surface_normal(x, z, c.nx, c.nz, c.mapscale, h);
    float* o = out + 12 * i;
    o[0] = (float)x; o[1] = py; o[2] = (float)z;
    o[3] = nv.x; o[4] = nv.y; o[5] = nv.z;
    o[6] = (float)(x + 1) - (float)x; o[7] = c.mapscale * h(x + 1, z) - py; o[8] = (float)z - (float)z;
    o[9] = (float)x - (float)x; o[10] = c.mapscale * h(x, z + 1) - py; o[11] = (float)(z + 1) - (float)z;
  }
}

}  // namespace

void launch_vertices(const float* height, const Consts& c, float* out, cudaStream_t s) {
  const long n = (long)c.nx * c.nz;
  long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  k_vertices<<<(int)g, 256, 0, s>>>(height, c, out);
}

void launch_windmap(const Fields& F, long n, float* out_rgba, cudaStream_t s) {
  long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  k_windmap<<<(int)g, 256, 0, s>>>(F.f[2], F.f[3], F.f[4], n, reinterpret_cast<float4*>(out_rgba));
}

}  // namespace swe
