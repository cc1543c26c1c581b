// Stencil traits for the device kernels.
//
// Direction tables and weights follow the reference's stencil files exactly
// (orderings differ between stencils):
//   D2Q9  stencils/D2Q9.cpp:40-61
//   D3Q19 stencils/D3Q19.cpp:37-67
//   D3Q27 stencils/D3Q27.cpp:36-112
// Unit (unscaled) velocities; the scaled velocity is scaling * e.
// dcls(i, a) is the index of the per-axis displacement class of direction i
// on axis a (-1: no displacement), used to select the streaming tables.
#pragma once

#include "natgpu_common.h"

namespace natgpu {

struct SD2Q9 {
  static constexpr int ID = 0, D = 2, Q = 9;
  __host__ __device__ static constexpr int e(int i, int a) {
    constexpr int E[9][3] = {{0, 0, 0},  {1, 0, 0},  {0, 1, 0},
                             {-1, 0, 0}, {0, -1, 0}, {1, 1, 0},
                             {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0}};
    return E[i][a];
  }
  __host__ __device__ static constexpr double w(int i) {
    return i == 0 ? 4. / 9. : (i <= 4 ? 1. / 9. : 1. / 36.);
  }
  __host__ __device__ static constexpr int dcls(int i, int a) {
    return e(i, a) > 0 ? 0 : (e(i, a) < 0 ? 1 : -1);
  }
};

struct SD3Q19 {
  static constexpr int ID = 1, D = 3, Q = 19;
  __host__ __device__ static constexpr int e(int i, int a) {
    constexpr int E[19][3] = {
        {0, 0, 0},  {1, 0, 0},  {0, 0, 1},  {-1, 0, 0}, {0, 0, -1},
        {0, -1, 0}, {0, 1, 0},  {1, 0, 1},  {-1, 0, 1}, {-1, 0, -1},
        {1, 0, -1}, {1, -1, 0}, {1, 1, 0},  {-1, 1, 0}, {-1, -1, 0},
        {0, -1, 1}, {0, 1, 1},  {0, 1, -1}, {0, -1, -1}};
    return E[i][a];
  }
  __host__ __device__ static constexpr double w(int i) {
    return i == 0 ? 1. / 3. : (i <= 6 ? 1. / 18. : 1. / 36.);
  }
  __host__ __device__ static constexpr int dcls(int i, int a) {
    return e(i, a) > 0 ? 0 : (e(i, a) < 0 ? 1 : -1);
  }
};

struct SD3Q27 {
  static constexpr int ID = 2, D = 3, Q = 27;
  __host__ __device__ static constexpr int e(int i, int a) {
    constexpr int E[27][3] = {
        {0, 0, 0},    {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},
        {0, 0, 1},    {0, 0, -1},  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},
        {0, -1, 1},   {1, 0, 1},   {-1, 0, -1}, {1, 0, -1},  {-1, 0, 1},
        {1, 1, 0},    {-1, -1, 0}, {1, -1, 0},  {-1, 1, 0},  {1, 1, 1},
        {-1, -1, -1}, {1, 1, -1},  {-1, -1, 1}, {1, -1, 1},  {-1, 1, -1},
        {1, -1, -1},  {-1, 1, 1}};
    return E[i][a];
  }
  __host__ __device__ static constexpr double w(int i) {
    return i == 0 ? 8. / 27.
                  : (i <= 6 ? 2. / 27. : (i <= 18 ? 1. / 54. : 1. / 216.));
  }
  __host__ __device__ static constexpr int dcls(int i, int a) {
    return e(i, a) > 0 ? 0 : (e(i, a) < 0 ? 1 : -1);
  }
};

// compile-time loop helper
template <int I>
struct IC {
  static constexpr int value = I;
};
template <int B, int E, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (B < E) {
    f(IC<B>{});
    static_for<B + 1, E>(f);
  }
}

}  // namespace natgpu
