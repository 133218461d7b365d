// Element functions of the medium packing (grids -> 64-byte lookup cells,
// albedo state pairs, majorants), of the per-pixel sample reduction and of
// the gradient fold (cell gradients -> voxel gradients), shared by the
// single-job and the batched kernels.
#pragma once
#include "rcv_volume.cuh"

namespace rcv {

// Cell i of a (dx+1)(dy+1)(dz+1) lattice: the 8 clamped corner voxels of the
// old and the new density.
// 32-bit index arithmetic: 4 (dx+1)(dy+1)(dz+1) < 2^32 is enforced on the host.
__device__ __forceinline__ void pack_cell(int64_t i, int dx, int dy, int dz, const float* __restrict__ old_d,
                                          const float* __restrict__ new_d, float4* __restrict__ cells) {
  const uint32_t ex = (uint32_t)(dx + 1), ey = (uint32_t)(dy + 1);
  const uint32_t row = (uint32_t)i / ex;
  const int cx = int((uint32_t)i - row * ex);
  const uint32_t cz_u = row / ey;
  const int cy = int(row - cz_u * ey);
  const int cz = int(cz_u);
  const int x0 = clampi(cx - 1, dx - 1), x1 = clampi(cx, dx - 1);
  const int y0 = clampi(cy - 1, dy - 1), y1 = clampi(cy, dy - 1);
  const int z0 = clampi(cz - 1, dz - 1), z1 = clampi(cz, dz - 1);
  auto idx = [&](int x, int y, int z) { return (int64_t(z) * dy + y) * dx + x; };
  const int64_t i000 = idx(x0, y0, z0), i100 = idx(x1, y0, z0), i010 = idx(x0, y1, z0), i110 = idx(x1, y1, z0),
                i001 = idx(x0, y0, z1), i101 = idx(x1, y0, z1), i011 = idx(x0, y1, z1), i111 = idx(x1, y1, z1);
  float4* c = cells + i * 4;
  c[0] = make_float4(old_d[i000], old_d[i100], old_d[i010], old_d[i110]);
  c[1] = make_float4(old_d[i001], old_d[i101], old_d[i011], old_d[i111]);
  c[2] = make_float4(new_d[i000], new_d[i100], new_d[i010], new_d[i110]);
  c[3] = make_float4(new_d[i001], new_d[i101], new_d[i011], new_d[i111]);
}

// Voxels whose trilinear weight can be non-zero inside supergrid cell c of
// S cells along an axis of D voxels: x in [c/S, (c+1)/S) reads voxels
// floor(xD - 1/2) and floor(xD - 1/2) + 1, clamped to [0, D-1].
__device__ __forceinline__ void supergrid_span(int c, int S, int D, int& lo, int& hi) {
  const int64_t a = 2 * int64_t(c) * D - S, b = 2 * int64_t(c + 1) * D - S, den = 2 * int64_t(S);
  const int64_t fa = a >= 0 ? a / den : -((-a + den - 1) / den);  // floor division
  const int64_t fb = b >= 0 ? b / den : -((-b + den - 1) / den);
  lo = clampi((int)fa, D - 1);
  hi = clampi((int)fb + 1, D - 1);
}

// Majorants of supergrid cell i (x fastest): scale * the largest old / new
// density (non-negative part) over its voxel span; two = max of both states.
__device__ __forceinline__ void supergrid_cell(int64_t i, const int sg[3], int dx, int dy, int dz, float scale,
                                               const float* __restrict__ old_d, const float* __restrict__ new_d,
                                               float* __restrict__ sg_two, float* __restrict__ sg_new) {
  const int cx = int(i % sg[0]), cy = int((i / sg[0]) % sg[1]), cz = int(i / (int64_t(sg[0]) * sg[1]));
  int x0, x1, y0, y1, z0, z1;
  supergrid_span(cx, sg[0], dx, x0, x1);
  supergrid_span(cy, sg[1], dy, y0, y1);
  supergrid_span(cz, sg[2], dz, z0, z1);
  float mo = 0.0f, mn = 0.0f;
  for (int z = z0; z <= z1; ++z)
    for (int y = y0; y <= y1; ++y)
      for (int x = x0; x <= x1; ++x) {
        const int64_t v = (int64_t(z) * dy + y) * dx + x;
        mo = fmaxf(mo, old_d[v]);
        mn = fmaxf(mn, new_d[v]);
      }
  sg_two[i] = scale * fmaxf(mo, mn);
  sg_new[i] = scale * mn;
}

// Voxel i of the old and the new RGB albedo as one 32-byte pair.
__device__ __forceinline__ void pack_albedo(int64_t i, const float* __restrict__ old_a,
                                            const float* __restrict__ new_a, float4* __restrict__ albedo) {
  albedo[i * 2 + 0] = make_float4(old_a[i * 3 + 0], old_a[i * 3 + 1], old_a[i * 3 + 2], 0.0f);
  albedo[i * 2 + 1] = make_float4(new_a[i * 3 + 0], new_a[i * 3 + 1], new_a[i * 3 + 2], 0.0f);
}

// Sum of a pixel's per-path radiance slots in sample order, divided by spp
// (the box-filter film develop of plugins/twostatevolpath.py:80-89).  Slots
// are [path][new, old] for two-state launches and [path] otherwise.
template <bool kTwo>
__device__ __forceinline__ void reduce_pixel(const float4* __restrict__ path_out, int64_t path_begin, int64_t pix,
                                             int spp, V3& out_new, V3& out_old) {
  constexpr int K = kTwo ? 2 : 1;
  const float4* src = path_out + (path_begin + pix * spp) * K;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f, ox = 0.0f, oy = 0.0f, oz = 0.0f;
  for (int s = 0; s < spp; ++s) {
    const float4 a = __ldcs(src + s * K);
    nx += a.x;
    ny += a.y;
    nz += a.z;
    if (kTwo) {
      const float4 b = __ldcs(src + s * K + 1);
      ox += b.x;
      oy += b.y;
      oz += b.z;
    }
  }
  const float fs = (float)spp;
  out_new = V3{nx / fs, ny / fs, nz / fs};
  out_old = V3{ox / fs, oy / fs, oz / fs};
}

// Block-wide max of the voxel densities into maxbits[0] (old), [1] (new);
// every thread of the block must call it (blockDim a multiple of 32).
// Non-negative floats order like their bits.  One atomicMax per block and
// state, skipped when the word already holds at least the block's value:
// every value it ever holds is the maximum of some voxels, so a smaller one
// cannot change the result, and a stale read only costs an unneeded atomic.
// (Per-warp atomics on the same two words serialised in one L2 slice and
// took most of a 128^3 grid's packing time.)
__device__ __forceinline__ void reduce_majorants(float mo, float mn, uint32_t* maxbits) {
  __shared__ uint32_t s_max[2][32];
  uint32_t bo = __float_as_uint(fmaxf(mo, 0.0f)), bn = __float_as_uint(fmaxf(mn, 0.0f));
  bo = __reduce_max_sync(0xffffffffu, bo);
  bn = __reduce_max_sync(0xffffffffu, bn);
  const unsigned w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_max[0][w] = bo;
    s_max[1][w] = bn;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const unsigned nw = (blockDim.x + 31) >> 5;
    bo = threadIdx.x < nw ? s_max[0][threadIdx.x] : 0u;
    bn = threadIdx.x < nw ? s_max[1][threadIdx.x] : 0u;
    bo = __reduce_max_sync(0xffffffffu, bo);
    bn = __reduce_max_sync(0xffffffffu, bn);
    if (threadIdx.x == 0) {
      if (bo != 0u && bo > __ldcg(maxbits + 0)) atomicMax(maxbits + 0, bo);
      if (bn != 0u && bn > __ldcg(maxbits + 1)) atomicMax(maxbits + 1, bn);
    }
  }
}

// Whether cell c of an axis of D voxels uses voxel v as its corner `bit`
// (corner 0 is voxel clamp(c - 1), corner 1 voxel clamp(c)).  Only cells v
// and v + 1 can, so a voxel has at most 4 (cell, bit) pairs per axis.
__device__ __forceinline__ bool fold_uses(int c, int bit, int v, int D) {
  return c <= D && clampi(c - 1 + bit, D - 1) == v;
}

// Gradient of voxel i: the sum of its corner entries in every cell that uses
// it, in the order z, y, x candidate, each by cell and then corner bit.  The
// candidate slots are fixed (cell v or v + 1, bit 0 or 1) and unrolled, so
// everything stays in registers.
__device__ __forceinline__ float fold_voxel(int64_t i, int dx, int dy, int dz, const float* __restrict__ gcells) {
  // 32-bit index arithmetic (the voxel count is below the cell count, < 2^30)
  const uint32_t row = (uint32_t)i / (uint32_t)dx;
  const int x = int((uint32_t)i - row * (uint32_t)dx);
  const uint32_t z_u = row / (uint32_t)dy;
  const int y = int(row - z_u * (uint32_t)dy), z = int(z_u);
  float g = 0.0f;
#pragma unroll
  for (int kz = 0; kz < 4; ++kz) {
    const int cz = z + (kz >> 1), bz = kz & 1;
    if (!fold_uses(cz, bz, z, dz)) continue;
#pragma unroll
    for (int ky = 0; ky < 4; ++ky) {
      const int cy = y + (ky >> 1), by = ky & 1;
      if (!fold_uses(cy, by, y, dy)) continue;
#pragma unroll
      for (int kx = 0; kx < 4; ++kx) {
        const int cx = x + (kx >> 1), bx = kx & 1;
        if (!fold_uses(cx, bx, x, dx)) continue;
        const int64_t cell = (int64_t(cz) * (dy + 1) + cy) * (dx + 1) + cx;
        g += gcells[cell * 8 + bx + 2 * by + 4 * bz];
      }
    }
  }
  return g;
}

// RGB gradient of albedo voxel i from the albedo cell records (24 floats per
// cell: corner k = bx + 2 by + 4 bz, then R, G, B), summed in the order of
// fold_voxel.
__device__ __forceinline__ V3 fold_voxel_rgb(int64_t i, int dx, int dy, int dz, const float* __restrict__ gcells) {
  const uint32_t row = (uint32_t)i / (uint32_t)dx;
  const int x = int((uint32_t)i - row * (uint32_t)dx);
  const uint32_t z_u = row / (uint32_t)dy;
  const int y = int(row - z_u * (uint32_t)dy), z = int(z_u);
  V3 g{0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int kz = 0; kz < 4; ++kz) {
    const int cz = z + (kz >> 1), bz = kz & 1;
    if (!fold_uses(cz, bz, z, dz)) continue;
#pragma unroll
    for (int ky = 0; ky < 4; ++ky) {
      const int cy = y + (ky >> 1), by = ky & 1;
      if (!fold_uses(cy, by, y, dy)) continue;
#pragma unroll
      for (int kx = 0; kx < 4; ++kx) {
        const int cx = x + (kx >> 1), bx = kx & 1;
        if (!fold_uses(cx, bx, x, dx)) continue;
        const int64_t cell = (int64_t(cz) * (dy + 1) + cy) * (dx + 1) + cx;
        const float* r = gcells + cell * 24 + (bx + 2 * by + 4 * bz) * 3;
        g = V3{g.x + r[0], g.y + r[1], g.z + r[2]};
      }
    }
  }
  return g;
}

}  // namespace rcv
