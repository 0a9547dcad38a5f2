// lca_common.cuh -- geometry and threshold shared by the tensor-core and FP32 forms of the
// batched LCA solver (lca_solver.cu, lca_solver_fp32.cu).
#pragma once

#include "pvgpu_internal.cuh"

#include <cfloat>

namespace pvgpu {

// V1 (nb images x v1Ny x v1Nx positions x F features) over an error/input layer of
// inNy x inNx x C pixels, stride S = inNx / v1Nx, square patch P (one-to-many,
// PatchGeometry::calcPatchStartInPost: patch start = S*y - (P - S)/2).
struct LcaGeom {
   int nb;
   int inNx, inNy;
   int v1Nx, v1Ny, F;
   int Npos, MB, rowsPerBlock;  // positions per image, 128-position blocks per image, V1 rows per block
   int NT;                      // feature tile of the post kernel
   float VThresh, AMin, AMax, AShift, VWidth;
   float e, si;                 // decay factor (float)exp(-dt/tau), selfInteract
   int simple;                  // AMax = +inf and VWidth = 0: A = V < VThresh ? AMin : V - AShift
};

// Device layout of the membrane potential V (solver-internal; the state and reset entry points
// convert to and from the reference's [nb][ny][nx][nf]): one 32 KB chunk per (image, block of
// 128 positions, block of 64 features), chunks in that order, so an image's chunks are
// contiguous.  Inside a chunk: two halves of 32 features, each 128 rows (positions) of 128 B,
// the 16-byte group j of row r stored at group j ^ (r % 8) -- the 128-byte swizzle, so that a
// chunk copied linearly into 1024-byte aligned shared memory is conflict-free to read by rows.
__host__ __device__ inline size_t v_index(const LcaGeom &g, int b, int pos, int f) {
   const int mb = pos >> 7, r = pos & 127, fb = f >> 6, h = (f >> 5) & 1, j = (f >> 2) & 7, e = f & 3;
   const size_t chunk = ((size_t)b * g.MB + mb) * (size_t)(g.F >> 6) + fb;
   return chunk * 8192 + (size_t)h * 4096 + (size_t)r * 32 + (size_t)((j ^ (r & 7)) << 2) + e;
}

// ANNActivityBuffer::applyVThresh / applyAMax (components/ANNActivityBuffer.cpp:490-558)
__device__ __forceinline__ float lca_thresh(float v, const LcaGeom &g) {
   float a = v;
   if (g.VThresh > -FLT_MAX) {
      float vtw = __fadd_rn(g.VThresh, g.VWidth);
      if (v < g.VThresh) a = g.AMin;
      else if (v < vtw) {
         float c = __fadd_rn(__fadd_rn(vtw, -g.AShift), -g.AMin);
         a = __fadd_rn(g.AMin, __fdiv_rn(__fmul_rn(c, __fadd_rn(v, -g.VThresh)), g.VWidth));
      } else a = __fadd_rn(a, -g.AShift);
   }
   if (g.AMax < FLT_MAX && a > g.AMax) a = g.AMax;
   return a;
}

// Residual window of a 128-position block: error rows [S*y0 - E, +rows), cols [-E, +cols).
__host__ __device__ inline int rwin_rows(int S, int P, int rowsPerBlock) { return S * (rowsPerBlock - 1) + P; }
__host__ __device__ inline int rwin_cols(int S, int P, int v1Nx) { return S * (v1Nx - 1) + P; }

// r = x - (sum of the image's partial reconstructions, in block order) over the window;
// zero outside the restricted error layer (its halo is zero).
template <int S, int P, int C, int NTHREADS>
__device__ __forceinline__ void build_residual_window(const LcaGeom &g, int b, int mb, const float *__restrict__ x,
                                                      const float *__restrict__ partials, float *rwin) {
   constexpr int E = (P - S) / 2;
   const int RWR = rwin_rows(S, P, g.rowsPerBlock), RWC = rwin_cols(S, P, g.v1Nx);
   const int y0 = mb * g.rowsPerBlock;
   const int nPix = g.inNx * g.inNy * C;
   const float *xb = x + (size_t)b * nPix;
   const float *pb = partials + (size_t)b * g.MB * nPix;
   for (int i = threadIdx.x; i < RWR * RWC * C; i += NTHREADS) {
      const int c = i % C, xr = (i / C) % RWC, yr = i / (C * RWC);
      const int ye = S * y0 - E + yr, xe = -E + xr;
      float v = 0.0f;
      if (ye >= 0 && ye < g.inNy && xe >= 0 && xe < g.inNx) {
         const int pi = (ye * g.inNx + xe) * C + c;
         float rec = pb[pi];
         for (int m = 1; m < g.MB; m++) rec = __fadd_rn(rec, pb[(size_t)m * nPix + pi]);
         v = __fadd_rn(xb[pi], -rec);
      }
      rwin[i] = v;
   }
}

}  // namespace pvgpu
