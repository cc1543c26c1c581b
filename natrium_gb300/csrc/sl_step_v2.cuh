// Fused semi-Lagrangian stream + collide, specialised kernel.
//
// Same operator as k_sl_step (sl_step.cuh), specialised at compile time on
// the FE order P, the node topology (FE_Q / DG) and the tile shape in cells,
// for the common case where every departure point lies in the node's own
// cell or in the adjacent upwind cell (the host checks this; CFL <= 1 with
// respect to the Gauss-Lobatto spacing).  Then, per axis and displacement
// sign, the 1-D factor of an output cell k only reads the source block that
// starts at node k * PER of the source region, and every node class reads at
// a compile-time offset inside that block.
//
// Pipeline per CTA (one tile of CX x CY x CZ cells):
//   * the source region of direction alpha + 1 is copied HBM/L2 -> shared
//     memory with bulk asynchronous copies (cp.async.bulk, one per region
//     row, 16-byte aligned; a row that crosses the periodic boundary is split
//     into two aligned segments) completing on an mbarrier, while direction
//     alpha is being computed (double buffer);
//   * the 1-D factors run cell by cell: a thread loads the 2 PER (or 2P+1)
//     values of one source block once and produces the PER outputs of the
//     cell, with the weights in the kernel's constant bank;
//   * the last factor writes the streamed population into a shared-memory
//     buffer [Q][tile nodes]; after the last direction each thread collides
//     its nodes from that buffer and writes f once, coalesced along x.
// In the FP32 deviation mode the streamed value is evaluated as
//   v_j0 + sum_{j != j0} W_j (v_j - v_j0),
// j0 being the source node at the destination node's own position (the
// dominant weight): a constant field is reproduced exactly whatever the float
// rounding of the weights, and that rounding only multiplies the small
// differences, so it adds no bias to mass or momentum.
#pragma once

#include <cuda_runtime.h>

#include "collision.cuh"
#include "natgpu_common.h"
#include "stencils.cuh"

namespace natgpu {

// Weights of the specialised kernel, passed by value (constant bank).
// [axis][sign: 0 -> e > 0, 1 -> e < 0][class][j]
template <class Real>
struct SpecWeights {
  Real w[3][2][PER_MAX][PMAX1];
};

template <class Real>
struct StepParams2 {
  const Real* f_in;
  Real* f_out;
  double* rho;
  double* u;
  int* status;
  long long n;
  int nx, ny, nz;
  int ntx, nty;
  double tau;
  double scaling;
  int write_macro;
  unsigned wait_polls;  // limit of each wait for a region copy (MBAR_MAX_POLLS)
  SpecWeights<Real> W;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// ---- bulk asynchronous copies and mbarriers --------------------------------
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst_smem, const void* src, unsigned bytes,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_u32(dst_smem)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Wait for the phase with the given parity; bounded: returns false after
// max_polls unsuccessful polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned max_polls) {
  for (unsigned it = 0; it < max_polls; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// status bit of a wait that ran out (the kernel then stops the tile)
constexpr int ST_TIMEOUT = 4;
constexpr unsigned MBAR_MAX_POLLS = 1u << 24;

template <int P, bool DG>
struct Geo {
  static constexpr int PER = DG ? P + 1 : P;
  // source region extent for displacement sign s (0: none, +1, -1) along an
  // axis whose tile extent is B
  __host__ __device__ static constexpr int R(int B, int s) {
    return s == 0 ? B : (s > 0 ? B + P + 1 : (DG ? B + P + 1 : B + 1));
  }
  // region start relative to the tile start
  __host__ __device__ static constexpr int RS(int s) { return s > 0 ? -PER : 0; }
  // window length of one output cell
  __host__ __device__ static constexpr int WIN(int s) {
    return s > 0 ? PER + P + 1 : (DG ? PER + P + 1 : P + 1);
  }
  // offset of class c's window inside the cell's window
  __host__ __device__ static constexpr int OFF(int s, int c) {
    return s > 0 ? (c == 0 ? 0 : PER) : ((DG && c == P) ? PER : 0);
  }
  // 16-byte aligned row segment in elements of size ES: start offset
  // (relative to the tile start, which is ALIGN-aligned), width, and the
  // column of the region start inside the row
  __host__ __device__ static constexpr int fl(int a, int m) { return a >= 0 ? a / m * m : -((-a + m - 1) / m) * m; }
  __host__ __device__ static constexpr int ce(int a, int m) { return -fl(-a, m); }
  __host__ __device__ static constexpr int XS(int B, int s, int m) { return fl(RS(s), m); }
  __host__ __device__ static constexpr int XW(int B, int s, int m) { return ce(RS(s) + R(B, s), m) - fl(RS(s), m); }
  __host__ __device__ static constexpr int XC(int B, int s, int m) { return RS(s) - fl(RS(s), m); }
  // index inside class c's window of the source node at the destination's
  // own position (the dominant weight)
  __host__ __device__ static constexpr int J0(int s, int c) {
    return s > 0 ? (c == 0 ? P : c) : ((DG && c == P) ? 0 : c);
  }
};

// odd row pitch for conflict-free strided access
__host__ __device__ constexpr int odd(int x) { return x | 1; }

template <class S, int P, bool DG, int CX, int CY, int CZ, int ES>
struct Tile {
  using G = Geo<P, DG>;
  static constexpr int PER = G::PER;
  static constexpr int D = S::D;
  static constexpr int AL = 16 / ES;  // elements per 16 bytes
  static constexpr int BX = CX * PER;
  static constexpr int BY = CY * PER;
  static constexpr int BZ = D == 3 ? CZ * PER : 1;
  static constexpr int TB = BX * BY * BZ;
  static constexpr int RYM = BY + P + 1, RZM = D == 3 ? BZ + P + 1 : 1;
  static constexpr int mx(int a, int b) { return a > b ? a : b; }
  static constexpr int PXM = mx(mx(G::XW(BX, 1, AL), G::XW(BX, -1, AL)), G::XW(BX, 0, AL));
  static constexpr int REGION = PXM * RYM * RZM;  // one region buffer (elements)
  static constexpr int T1 = PXM * RYM * BZ;       // output of a first (non-final) stage
  static constexpr int T2 = PXM * BY * BZ;        // output of a second (non-final) stage
  // most factors any direction needs (3 only for the corner directions of D3Q27)
  static constexpr int maxstages() {
    int m = 0;
    for (int i = 1; i < S::Q; ++i) {
      int k = (S::e(i, 0) != 0) + (S::e(i, 1) != 0) + (D == 3 && S::e(i, 2) != 0);
      m = k > m ? k : m;
    }
    return m;
  }
  static constexpr int NSTAGE = maxstages();
  static constexpr int NREG = 3;  // region buffers in flight
  static constexpr size_t ELEMS = (size_t)NREG * REGION + (NSTAGE >= 2 ? 2 * (size_t)T1 : 0) +
                                  (NSTAGE >= 3 ? 2 * (size_t)T2 : 0) + (size_t)S::Q * TB;
  static_assert(BX % AL == 0, "tile x extent must keep 16-byte row alignment");
};

template <class S, class Real, int P, bool DG, int CX, int CY, int CZ>
__host__ __device__ constexpr size_t v2_smem_bytes() {
  using TL = Tile<S, P, DG, CX, CY, CZ, sizeof(Real)>;
  return 128 + sizeof(Real) * TL::ELEMS;
}

// ---------------------------------------------------------------------------
// One 1-D factor.  Input box (IX, IY, IZ) with row pitch IP; output box with
// the extent along axis A replaced by CA * PER, row pitch OP.  Work item =
// (line perpendicular to A, output cell along A).
// ---------------------------------------------------------------------------
template <int A, int SG, class Real, int P, bool DG, bool DEV, int CA, int IX, int IY, int IZ, int IP, int OP,
          int NTH>
__device__ __forceinline__ void factor(const Real* __restrict__ in, Real* __restrict__ out,
                                       const Real (&W)[PER_MAX][PMAX1]) {
  using G = Geo<P, DG>;
  constexpr int PER = G::PER;
  constexpr int WIN = G::WIN(SG);
  constexpr int OX = A == 0 ? CA * PER : IX;
  constexpr int OY = A == 1 ? CA * PER : IY;
  constexpr int OZ = A == 2 ? CA * PER : IZ;
  // lines: the two axes other than A
  constexpr int L0 = A == 0 ? IY : IX;  // fastest line index
  constexpr int L1 = A == 2 ? IY : IZ;
  constexpr int NLINE = L0 * L1;
  constexpr int NWORK = NLINE * CA;
  constexpr int sIn = A == 0 ? 1 : (A == 1 ? IP : IP * IY);
  constexpr int sOut = A == 0 ? 1 : (A == 1 ? OP : OP * OY);
  (void)OX;
  (void)OZ;
  for (int w = threadIdx.x; w < NWORK; w += NTH) {
    // x factor: cells fastest across lanes (stride PER, conflict-free);
    // y / z factors: lines (consecutive x) fastest
    const int line = A == 0 ? w / CA : w % NLINE;
    const int k = A == 0 ? w % CA : w / NLINE;
    const int l0 = line % L0;
    const int l1 = line / L0;
    int bi, bo;  // base offsets of the line
    if constexpr (A == 0) {
      bi = (l1 * IY + l0) * IP;
      bo = (l1 * OY + l0) * OP;
    } else if constexpr (A == 1) {
      bi = l1 * IY * IP + l0;
      bo = l1 * OY * OP + l0;
    } else {
      bi = l1 * IP + l0;
      bo = l1 * OP + l0;
    }
    const Real* src = in + bi + (k * PER) * sIn;
    Real v[WIN];
#pragma unroll
    for (int j = 0; j < WIN; ++j) v[j] = src[j * sIn];
    Real* dst = out + bo + (k * PER) * sOut;
#pragma unroll
    for (int c = 0; c < PER; ++c) {
      const int o = G::OFF(SG, c);
      Real acc;
      if constexpr (DEV) {
        const int j0 = G::J0(SG, c);
        const Real v0 = v[o + j0];
        acc = Real(0);
#pragma unroll
        for (int j = 0; j <= P; ++j)
          if (j != j0) acc = fma(W[c][j], v[o + j] - v0, acc);
        acc += v0;
      } else {
        acc = W[c][0] * v[o];
#pragma unroll
        for (int j = 1; j <= P; ++j) acc = fma(W[c][j], v[o + j], acc);
      }
      dst[c * sOut] = acc;
    }
  }
}

// Issue the bulk copies of one direction's source region (one or two per
// row) completing on bar; thread 0 registers the byte count.
template <class S, class Real, int P, bool DG, int CX, int CY, int CZ, int ALPHA, int NTH>
__device__ __forceinline__ void load_region(const Real* __restrict__ src, Real* buf, unsigned long long* bar,
                                            int x0, int y0, int z0, int nx, int ny, int nz) {
  using TL = Tile<S, P, DG, CX, CY, CZ, sizeof(Real)>;
  using G = Geo<P, DG>;
  constexpr int AL = TL::AL;
  constexpr int sx = S::e(ALPHA, 0), sy = S::e(ALPHA, 1), sz = TL::D == 3 ? S::e(ALPHA, 2) : 0;
  constexpr int RY = G::R(TL::BY, sy), RZ = TL::D == 3 ? G::R(TL::BZ, sz) : 1;
  constexpr int XW = G::XW(TL::BX, sx, AL);
  constexpr int ROWS = RY * RZ;
  constexpr unsigned BYTES = (unsigned)(ROWS * XW * sizeof(Real));
  if (threadIdx.x == 0) mbar_expect_tx(bar, BYTES);
  const int xs = x0 + G::XS(TL::BX, sx, AL);  // aligned row start (may be < 0 or run past nx)
  const int gy0 = y0 + G::RS(sy), gz0 = z0 + G::RS(sz);
  for (int r = threadIdx.x; r < ROWS; r += NTH) {
    const int y = r % RY, z = r / RY;
    int gy = gy0 + y, gz = gz0 + z;
    gy += gy < 0 ? ny : 0;
    gy -= gy >= ny ? ny : 0;
    gz += gz < 0 ? nz : 0;
    gz -= gz >= nz ? nz : 0;
    const Real* row = src + ((long long)gz * ny + gy) * nx;
    Real* dst = buf + (z * RY + y) * TL::PXM;
    // periodic row segment [xs, xs + XW): at most three aligned pieces
    int done = 0;
    int pos = xs < 0 ? xs + nx : xs;
#pragma unroll 1
    for (int piece = 0; piece < 4 && done < XW; ++piece) {
      const int len = min(XW - done, nx - pos);
      bulk_copy(dst + done, row + pos, (unsigned)(len * sizeof(Real)), bar);
      done += len;
      pos = 0;
    }
  }
}

// Per direction: its factors in the order z, y, x (active axes only) and the
// box extents before each of them.
template <class S, int P, bool DG, int CX, int CY, int CZ, int ES, int ALPHA>
struct Dir {
  using TL = Tile<S, P, DG, CX, CY, CZ, ES>;
  using G = Geo<P, DG>;
  static constexpr int sx = S::e(ALPHA, 0), sy = S::e(ALPHA, 1), sz = TL::D == 3 ? S::e(ALPHA, 2) : 0;
  static constexpr int NS = (sz != 0) + (sy != 0) + (sx != 0);
  static constexpr int RX = G::R(TL::BX, sx), RY = G::R(TL::BY, sy), RZ = TL::D == 3 ? G::R(TL::BZ, sz) : 1;
  // axis of stage k
  static constexpr int axis(int k) {
    int a[3] = {0, 0, 0}, n = 0;
    if (sz != 0) a[n++] = 2;
    if (sy != 0) a[n++] = 1;
    if (sx != 0) a[n++] = 0;
    return a[k];
  }
  // extent along axis b before stage k (factors before k have reduced
  // their axis to the tile extent)
  static constexpr int ext(int k, int b) {
    int e = b == 0 ? RX : (b == 1 ? RY : RZ);
    for (int j = 0; j < k; ++j)
      if (axis(j) == b) e = b == 0 ? TL::BX : (b == 1 ? TL::BY : TL::BZ);
    return e;
  }
  static constexpr int sign(int b) { return b == 0 ? sx : (b == 1 ? sy : sz); }
  static constexpr int cells(int b) { return b == 0 ? CX : (b == 1 ? CY : CZ); }
  static constexpr int XC = G::XC(TL::BX, sx, TL::AL);  // column of the region x origin
};

// Stage K of direction ALPHA: reads the region (K = 0) or the previous
// stage's buffer, writes the next stage buffer or (last stage) the streamed
// buffer.
template <class S, class Real, int P, bool DG, bool DEV, int CX, int CY, int CZ, int ALPHA, int K, int NTH>
__device__ __forceinline__ void run_stage(Real* const (&reg)[3], Real* const (&st1)[2], Real* const (&st2)[2],
                                          Real* sb, const SpecWeights<Real>& W) {
  using TL = Tile<S, P, DG, CX, CY, CZ, sizeof(Real)>;
  using DI = Dir<S, P, DG, CX, CY, CZ, sizeof(Real), ALPHA>;
  constexpr int A = DI::axis(K);
  constexpr int SG = DI::sign(A);
  constexpr int CA = DI::cells(A);
  constexpr int IX = DI::ext(K, 0), IY = DI::ext(K, 1), IZ = DI::ext(K, 2);
  constexpr bool LAST = K == DI::NS - 1;
  constexpr int IP = TL::PXM;
  constexpr int OP = LAST ? TL::BX : TL::PXM;
  constexpr int sidx = SG > 0 ? 0 : 1;
  const Real* in;
  if constexpr (K == 0)
    in = reg[(ALPHA - 1) % 3] + DI::XC;
  else if constexpr (K == 1)
    in = st1[(ALPHA - 1) % 2] + DI::XC;
  else
    in = st2[(ALPHA - 1) % 2] + DI::XC;
  Real* out;
  if constexpr (LAST)
    out = sb + ALPHA * TL::TB;
  else if constexpr (K == 0)
    out = st1[(ALPHA - 1) % 2] + DI::XC;
  else
    out = st2[(ALPHA - 1) % 2] + DI::XC;
  factor<A, SG, Real, P, DG, DEV, CA, IX, IY, IZ, IP, OP, NTH>(in, out, W.w[A][sidx]);
}

// Phase PH of the software pipeline: stage K of direction ALPHA runs in
// phase ALPHA - 1 + K, for every direction whose stage falls in this phase.
template <class S, class Real, int P, bool DG, bool DEV, int CX, int CY, int CZ, int PH, int NTH>
__device__ __forceinline__ void run_phase(Real* const (&reg)[3], Real* const (&st1)[2], Real* const (&st2)[2],
                                          Real* sb, const SpecWeights<Real>& W) {
  static_for<0, 3>([&](auto KK) {
    constexpr int K = decltype(KK)::value;
    constexpr int ALPHA = PH + 1 - K;
    if constexpr (ALPHA >= 1 && ALPHA < S::Q) {
      using DI = Dir<S, P, DG, CX, CY, CZ, sizeof(Real), ALPHA>;
      if constexpr (K < DI::NS) run_stage<S, Real, P, DG, DEV, CX, CY, CZ, ALPHA, K, NTH>(reg, st1, st2, sb, W);
    }
  });
}

// MINB: resident CTAs per SM the register allocation is sized for (small
// tiles run several CTAs per SM, so that one computes while another waits at
// a barrier).
template <class S, class Real, int COLL, int P, bool DG, int CX, int CY, int CZ, int NTH, int MINB = 1>
__global__ void __launch_bounds__(NTH, MINB) k_sl_step_v2(const __grid_constant__ StepParams2<Real> prm) {
  constexpr bool DEV = sizeof(Real) == 4;
  using TL = Tile<S, P, DG, CX, CY, CZ, sizeof(Real)>;
  constexpr int Q = S::Q;
  constexpr int BX = TL::BX, BY = TL::BY, BZ = TL::BZ, TB = TL::TB;
  extern __shared__ __align__(128) unsigned char smem_v2[];
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem_v2);  // 3 mbarriers
  __shared__ int s_abort;
  Real* base = reinterpret_cast<Real*>(smem_v2 + 128);
  Real* const reg[3] = {base, base + TL::REGION, base + 2 * TL::REGION};
  Real* stb = base + 3 * TL::REGION;
  Real* const st1[2] = {stb, stb + (TL::NSTAGE >= 2 ? TL::T1 : 0)};
  stb += TL::NSTAGE >= 2 ? 2 * TL::T1 : 0;
  Real* const st2[2] = {stb, stb + (TL::NSTAGE >= 3 ? TL::T2 : 0)};
  stb += TL::NSTAGE >= 3 ? 2 * TL::T2 : 0;
  Real* sb = stb;

  const int bid = blockIdx.x;
  const int tx = bid % prm.ntx, ty = (bid / prm.ntx) % prm.nty, tz = bid / (prm.ntx * prm.nty);
  const int x0 = tx * BX, y0 = ty * BY, z0 = tz * BZ;
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const long long n = prm.n;
  const long long nxy = (long long)nx * ny;

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  // prologue: regions of directions 1, 2, 3
  static_for<1, 4>([&](auto I) {
    constexpr int A = decltype(I)::value;
    if constexpr (A < Q)
      load_region<S, Real, P, DG, CX, CY, CZ, A, NTH>(prm.f_in + (long long)A * n, reg[(A - 1) % 3],
                                                      &bars[(A - 1) % 3], x0, y0, z0, nx, ny, nz);
  });
  // rest population: not streamed
  for (int t = threadIdx.x; t < TB; t += NTH) {
    const int x = t % BX, y = (t / BX) % BY, z = t / (BX * BY);
    sb[t] = prm.f_in[(long long)(z0 + z) * nxy + (long long)(y0 + y) * nx + (x0 + x)];
  }
  bool ok = true;
  // phases 0 .. Q: phase PH starts stage 0 of direction PH + 1
  static_for<0, Q + 1>([&](auto I) {
    constexpr int PH = decltype(I)::value;
    constexpr int A = PH + 1;  // direction whose region is consumed now
    if (!ok) return;
    if constexpr (A < Q) {
      if (!mbar_wait(&bars[(A - 1) % 3], ((A - 1) / 3) & 1, prm.wait_polls)) s_abort = 1;
    }
    __syncthreads();
    if (s_abort) {
      // copies still in flight: directions A .. max(A + 1, 3), issued and
      // not yet waited for; wait for them (bounded) before the CTA exits
      if constexpr (A < Q) {
        constexpr int HI = A + 1 > 3 ? A + 1 : 3;
        constexpr int LAST = HI < Q - 1 ? HI : Q - 1;
        if (threadIdx.x == 0)
          static_for<A, LAST + 1>([&](auto J) {
            constexpr int D = decltype(J)::value;
            mbar_wait(&bars[(D - 1) % 3], ((D - 1) / 3) & 1, MBAR_MAX_POLLS);
          });
      }
      ok = false;
      return;
    }
    // direction A + 2 shares its region buffer with direction A - 1, whose
    // region was last read in phase PH - 1 (before the barrier above)
    if constexpr (A + 2 < Q && PH >= 1)
      load_region<S, Real, P, DG, CX, CY, CZ, A + 2, NTH>(prm.f_in + (long long)(A + 2) * n, reg[(A + 1) % 3],
                                                          &bars[(A + 1) % 3], x0, y0, z0, nx, ny, nz);
    run_phase<S, Real, P, DG, DEV, CX, CY, CZ, PH, NTH>(reg, st1, st2, sb, prm.W);
  });
  if (!ok) {
    // a wait for a bulk copy ran out: report and stop this tile
    if (threadIdx.x == 0) atomicOr(prm.status, ST_TIMEOUT);
    return;
  }
  __syncthreads();

  // collision from the streamed buffer, one write of f
  int bad = 0;
  const Real inv_tau = Real(1) / Real(prm.tau);
  for (int t = threadIdx.x; t < TB; t += NTH) {
    Real v[Q], pre[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = sb[q * TB + t];
    Real u[3] = {0, 0, 0};
    Real rho = Real(1);
    if constexpr (DEV) {
#pragma unroll
      for (int q = 0; q < Q; ++q) pre[q] = v[q];
    }
    if constexpr (COLL == COLL_BGK) {
      rho = collide_bgk<S, DEV, false>(v, inv_tau, u, false);
      if constexpr (DEV) conserve<S>(v, pre);
    } else if constexpr (COLL == COLL_BGK_INC) {
      rho = collide_bgk_inc<DEV, false>(v, inv_tau, u, false);
    } else if constexpr (COLL == COLL_KBC) {
      rho = collide_kbc<S, DEV, false>(v, Real(prm.tau), u, false);
      if constexpr (DEV) conserve<S>(v, pre);
    }
    (void)pre;
    const int x = t % BX, y = (t / BX) % BY, z = t / (BX * BY);
    const long long node = (long long)(z0 + z) * nxy + (long long)(y0 + y) * nx + (x0 + x);
    if constexpr (COLL != COLL_NONE) {
      if (!(rho >= Real(1e-10))) bad |= (rho != rho) ? ST_NAN : ST_DENSITY;
      if (prm.write_macro) {
        prm.rho[node] = (double)rho;
        prm.u[node] = (double)u[0] * prm.scaling;
        prm.u[n + node] = (double)u[1] * prm.scaling;
        if constexpr (S::D == 3) prm.u[2 * n + node] = (double)u[2] * prm.scaling;
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) prm.f_out[(long long)q * n + node] = v[q];
  }
  if constexpr (COLL != COLL_NONE) {
    if (bad) atomicOr(prm.status, bad);
  }
}

}  // namespace natgpu
