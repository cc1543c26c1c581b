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

// D2Q25H (stencils/D2Q25H.cpp:37-84): the velocities are the products of the
// 1-D set {0, +-c_m, +-c_n}, c_m = sqrt(5 - sqrt 10) / sqrt 3 and
// c_n = sqrt(5 + sqrt 10) / sqrt 3 (unscaled); the weights are products of
// the 1-D weights.  The speeds themselves are not integers, so code(i, a)
// gives the component as a code (0 none, +-1 +-c_m, +-2 +-c_n); the values
// come from the host.  dcls(i, a): 0 +c_m, 1 -c_m, 2 +c_n, 3 -c_n, -1 none.
// group(i): the symmetry group (|code_x|, |code_y|) of the direction --
// (0,0) 0, (1,0) 1, (0,1) 2, (2,0) 3, (0,2) 4, (1,1) 5, (2,2) 6, (1,2) 7,
// (2,1) 8 -- whose members share |e_x|, |e_y| and the weight.
struct SD2Q25H {
  static constexpr int ID = 3, D = 2, Q = 25, NG = 9;
  __host__ __device__ static constexpr int code(int i, int a) {
    constexpr int C[25][2] = {{0, 0},  {1, 0},   {0, 1},   {-1, 0}, {0, -1}, {1, 1},   {-1, 1},
                              {-1, -1}, {1, -1}, {2, 0},   {0, 2},  {-2, 0}, {0, -2},  {2, 2},
                              {-2, 2}, {-2, -2}, {2, -2},  {1, 2},  {1, -2}, {-1, -2}, {-1, 2},
                              {2, 1},  {2, -1},  {-2, -1}, {-2, 1}};
    return C[i][a];
  }
  __host__ __device__ static constexpr int dcls(int i, int a) {
    return code(i, a) == 1 ? 0 : (code(i, a) == -1 ? 1 : (code(i, a) == 2 ? 2 : (code(i, a) == -2 ? 3 : -1)));
  }
  // sign of the component (+1 for none)
  __host__ __device__ static constexpr int sgn(int i, int a) { return code(i, a) < 0 ? -1 : 1; }
  __host__ __device__ static constexpr int group(int i) {
    constexpr int G[3][3] = {{0, 2, 4}, {1, 5, 7}, {3, 8, 6}};  // [|code_x|][|code_y|]
    return G[code(i, 0) < 0 ? -code(i, 0) : code(i, 0)][code(i, 1) < 0 ? -code(i, 1) : code(i, 1)];
  }
  // |code| per axis of a group
  __host__ __device__ static constexpr int gx(int g) {
    constexpr int X[9] = {0, 1, 0, 2, 0, 1, 2, 1, 2};
    return X[g];
  }
  __host__ __device__ static constexpr int gy(int g) {
    constexpr int Y[9] = {0, 0, 1, 0, 2, 1, 2, 2, 1};
    return Y[g];
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
