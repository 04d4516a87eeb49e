// Internal definition of the CISD_SO plan: dimensions, workspace carving and
// the device pointers of every block and per-iteration buffer.
#pragma once
#include "common.cuh"

struct agb_cisd_plan {
  int o, v, flags;
  int64_t nso, ov, po, pv, n1, n2;
  bool singles, mixed, f_diag, mp2_only;
  size_t ws_bytes;
  void* ws;
  // ---- static data (complex128 unless noted)
  agb::z64 *FvoT, *Foo, *Fvv, *EW;   // EW = [F_ov (ov) | <ij||ab> packed (n2)]
  double* eps;                        // nso SO orbital energies
  double* invD;                       // n1 + n2: 1 / D per amplitude (set with the orbital energies)
  int2 *opairs, *vpairs;              // packed pair -> (p,q)
  agb::z64 *R0p;                      // [po][pv] <ab||ij>
  agb::z64 *VT;                       // [(j,b)][(k,c)] <kb||cj>
  agb::z64 *WvovvH;                   // [a][j][p(cb)] <aj||cb>
  agb::z64 *WooovP;                   // [i][p(kj)][b] <kj||ib>
  agb::z64 *WovooP;                   // [p(ij)][b][k] <kb||ij>
  agb::z64 *WvvvoP;                   // [c][j][p(ab)] <ab||cj>
  agb::z64 *WooooT;                   // [p(ij)][p(kl)] <kl||ij>
  agb::z64 *Wvp;                      // [p(ab)][p(cd)] <ab||cd>
  // ---- per-iteration buffers
  agb::z64 *Tring;                    // [(i,a)][(k,c)] t2[i,k,a,c]
  agb::z64 *t2h;                      // [i][j][p(ab)]
  agb::z64 *t2q;                      // [p(ij)][a][b]
  agb::z64 *X;                        // [(i,a)][(j,b)] ring product
  agb::z64 *PQ;                       // [p(ij)][p(ab)] ladder products
  agb::z64 *Zq;                       // [p(ij)][b][a]
  agb::z64 *Yh;                       // [i][j][p(ab)]
  agb::z64 *Gq;                       // [p(ij)][a][b]
  agb::z64 *H2h;                      // [i][j][p(ab)]
  agb::z64 *R1x;                      // [(i,a)] sum_(k,c) t2[i,k,a,c] F_kc, from the ring-plane unpack
  // TF32 hi/lo planes of the static operands (mixed plans only)
  float *P_VT = nullptr, *P_Wvp = nullptr, *P_Woooo = nullptr, *P_Wvovv = nullptr, *P_Wooov = nullptr,
        *P_Wovoo = nullptr, *P_Wvvvo = nullptr;
  void* gemm_scratch;                 // 3xTF32 operand planes
  size_t gemm_scratch_bytes;
  // benchmark instrumentation: events around this plan's tcgen05 GEMM launches while on
  bool gemm_timing = false;
  agb::GemmTimingLog gemm_timing_log;
};
