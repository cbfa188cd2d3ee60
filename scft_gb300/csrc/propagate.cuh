// propagate.cuh -- batched FEM contour propagator + density (the hot path).
//
// One "group" of T = 32*NW threads owns one instance at a time; each thread owns
// C consecutive interior unknowns (a chunk).  Per field iterate the group
// assembles, in FP64, the implicit-Euler system D = M + ds(K + W) of
// 1D_FEM.c:95-186 (nonuniform mesh as Matlab_files/simple_FEM_1D_transient.m:34-85)
// and factors it once for the partition below; then it runs the nsteps contour
// steps of 1D_FEM.c:208-228 entirely on chip:
//
//   chunk level : Thomas sweep over the C-1 chunk-interior unknowns (registers),
//                 the last unknown of every chunk is its separator;
//   warp level  : the 32 chunk separators of a warp form a tridiagonal system,
//                 lanes 0..30 are solved by parallel cyclic reduction with warp
//                 shuffles, lane 31 is the warp separator;
//   group level : the NW warp separators form a tridiagonal system solved
//                 redundantly by every warp (PCR with shuffles); two named
//                 barriers per step exchange the warp-boundary values (on
//                 thread-block clusters: st.async stores completing on
//                 mbarriers, one exchange per step, see cx_*).
//
// The density phi_i = sum_k W_k q_k,i q_{nsteps-k},i (romint.c:21-57 Romberg
// weights, or the trapezoid of simple_FEM_1D_transient.m:119-124) is accumulated
// on the fly: slices k <= nsteps/2 are streamed coalesced to HBM, slices of the
// second half are multiplied against them as they are produced.
//
// FP32 path (DELTA = true): each step solves D dq = -ds (K+W) q for the small
// increment and adds it to q kept as an unevaluated float pair (hi + lo), so the
// per-step rounding scales with |dq| instead of |q|.  K q is formed from node
// differences of the pair, so it is exact on constants: FP32-rounded stiffness
// bands would not cancel and would bias every step by O(eps ds/h^2).  phi is
// Kahan-compensated.
// FP64 path (DELTA = false): the direct form D q' = M q of the reference.
#pragma once
#include <cooperative_groups.h>
#include <type_traits>

#include "common.cuh"
#include "mix_group.cuh"

namespace scft {

// Packed FP32 path: the (hi, lo) pairs are renormalised every PACKED_RENORM
// steps and density terms are summed in FP32 over PACKED_BLOCK steps before
// entering the Kahan total (both powers of two; 1 and 1 reproduce the rounding
// of a per-step two-sum and a per-step Kahan sum).
#ifndef PACKED_RENORM
#define PACKED_RENORM 1
#endif
#ifndef PACKED_BLOCK
#define PACKED_BLOCK 1
#endif
// Longest wait of a group for a claimed forked-path job to be published (ns).
#ifndef FORK_WAIT_NS
#define FORK_WAIT_NS 30000000000ull
#endif

// The second half of a contour pass reads back the slices the first half
// stored, one step ahead into registers.  Under load the slices come from HBM
// at a latency longer than a step, so each step of the packed FP32 loop in
// one-CTA groups also asks L2 for the slice it will read PREFETCH_STEPS steps
// later (prefetch.global.L2: no register).  Measured on the GB300: the
// warm-start evaluation classes' passes 7-13 % shorter; the cluster classes
// (graded meshes, barrier-bound) 7 % longer, so they do without; no change for
// the FP64 batch.
#ifndef PREFETCH_STEPS
#define PREFETCH_STEPS 4
#endif
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Minimum resident CTAs per SM the fused solve kernel is compiled for (its
// register budget); the planner sizes its grid from the occupancy it gets.
#ifndef SOLVE_MIN_CTAS
#define SOLVE_MIN_CTAS 1
#endif

template <typename R>
__device__ __forceinline__ R fmaR(R a, R b, R c);
template <>
__device__ __forceinline__ float fmaR<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ double fmaR<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

// hi + lo += d, exact sum of hi and d (Knuth two-sum) folded into lo, then renormalised.
__device__ __forceinline__ void ff_add(float &hi, float &lo, float d) {
  float s = __fadd_rn(hi, d);
  float bp = __fsub_rn(s, hi);
  float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(d, bp));
  float l = __fadd_rn(lo, e);
  float h = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(h, s));
  hi = h;
}

__device__ __forceinline__ void group_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <typename R, int NW>
struct GroupSmem {
  R pub_zc0[NW];  // per step, lane 0 of each warp: chunk-local z at its first unknown
  R pub_zw[NW];   // per step, lane 0 of each warp: warp-level interior solution
  R pub_R[NW];    // per step, lane 31 of each warp: level-2 right-hand side
  double s_vc0[NW], s_wc0[NW], s_vw0[NW], s_ww0[NW];
  double s_A[NW], s_B[NW], s_C[NW];
  double red[NW];
  int ired[NW];
  R qw[16];
  int item;
  // Cluster classes only: the per-step exchange between the CTAs of a cluster
  // (see cx_* below), double-buffered by step parity: every warp's A_w, zc0_w
  // and zw_w; per pass, every warp's coefficients of its level-2 right-hand
  // side on the next warp's values; the mbarriers the remote stores complete
  // on (parity 0, 1).
  R x_A[2][NW], x_Z0[2][NW], x_ZW[2][NW];
  R c_dus[NW], c_ga[NW];
  unsigned long long xbar[2];
  unsigned xk;  // exchange steps taken by this CTA (all instances so far)
  int xfail;    // a bounded exchange wait ran out (the cluster's results are void)
};

// Per-step exchange of the cluster classes.  Instead of two cluster barriers
// per contour step (each a release/acquire of the distributed-shared-memory
// stores by all CTAs), values move by st.async into every CTA's shared memory
// and complete on an mbarrier there (transaction bytes), so a CTA waits only
// for the bytes it reads, once per step.  Warp w's level-2 right-hand side is
// affine in the next warp's first-lane values:
//   R_w = A_w - dus_w zc0_{w+1} - ga_w zw_{w+1},  A_w = rl - dls zcl - al zw30
// (lane 31's terms), so each warp sends A_w, zc0_w and zw_w to every CTA and
// each lane l < NW forms R_l itself from the per-pass coefficients dus_l, ga_l.
// Ordering: a warp sends step k+1's values only after the step-k exchange of
// its own CTA completed, which needs every warp's step-k values, which each
// warp sends after reading its step-(k-1) inputs; so two buffers (step parity)
// suffice.  Each phase is armed (expected bytes) by thread 0 of the consumer
// CTA right after it saw the previous phase of that buffer complete, before
// its warp can send the values that let any warp reach the next use.  Every
// wait is bounded: after CX_WAIT_NS the thread marks every CTA of the cluster
// failed, and from then on the CTAs skip the exchange (no send, no wait, no
// arming), finish the same steps and report ST_WATCHDOG.
#ifndef CX_WAIT_NS
#define CX_WAIT_NS 1000000000ull
#endif
__device__ __forceinline__ unsigned cx_smem(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned cx_remote(unsigned a, int rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void cx_init(unsigned bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void cx_arm(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool cx_test(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void cx_send(unsigned raddr, float v, unsigned rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(raddr),
               "r"(__float_as_uint(v)), "r"(rbar)
               : "memory");
}
__device__ __forceinline__ void cx_send(unsigned raddr, double v, unsigned rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(raddr),
               "l"(__double_as_longlong(v)), "r"(rbar)
               : "memory");
}

template <int NW>
struct Log2 { static constexpr int v = NW <= 1 ? 0 : 1 + Log2<NW / 2>::v; };
template <>
struct Log2<1> { static constexpr int v = 0; };

// CL > 1: the group of one instance spans a thread-block cluster of CL CTAs of
// 32*NW/CL threads each (large shapes, whose 32*NW threads would otherwise get
// too few registers per thread in one CTA).  Group-level values are written to
// the shared memory of every CTA of the cluster (distributed shared memory) and
// read locally; outside the contour loop the group barrier is the cluster
// barrier, inside it the per-step exchange is st.async on mbarriers (cx_*).
template <typename R, int C, int NW, bool DELTA, int CL = 1>
struct Propagator {
  static constexpr int T = 32 * NW;
  static constexpr int TC = T * C;
  static constexpr int GPC = (CL > 1 || T >= 64) ? 1 : 64 / T;  // groups per CTA (small CTAs: occupancy is register-bound)
  static constexpr int CTA = (CL > 1) ? T / CL : T * GPC;
  static_assert(CL == 1 || (NW % CL == 0 && NW / CL >= 1), "cluster CTAs hold whole warps");
  static constexpr int L2 = Log2<NW>::v;
  static constexpr int CI = (C > 1) ? C - 1 : 1;       // chunk-interior array extent

  __device__ static void gsync(int bar_id) {
    if constexpr (CL > 1) cooperative_groups::this_cluster().sync();
    else if (NW > 1) group_sync(bar_id, T);
    else __syncwarp();
  }
  // store a group-level value where every thread of the group reads it
  template <typename V>
  __device__ static __forceinline__ void put(V &ref, V v) {
    if constexpr (CL > 1) {
      cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
#pragma unroll
      for (int r = 0; r < CL; r++) *cl.map_shared_rank(&ref, r) = v;
    } else {
      ref = v;
    }
  }

  __device__ static void run(const BatchDev &b, const ClassDev &cls, GroupSmem<R, NW> &S,
                             int P, int worker, int bar_id) {
    const int lane = P & 31, wid = P >> 5;
    R *slot = reinterpret_cast<R *>(cls.scratch) + (long long)worker * cls.slot_elems;
    for (;;) {
      int item;
      if (NW > 1) {
        if (P == 0) put(S.item, atomicAdd(cls.head, 1));
        gsync(bar_id);
        item = S.item;
        gsync(bar_id);
      } else {
        item = 0;
        if (lane == 0) item = atomicAdd(cls.head, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
      }
      if (item >= cls.count) break;
      const int inst = cls.items[item];
      if (b.active[inst] != cls.want) continue;
      instance(b, S, P, lane, wid, inst, slot, bar_id);
      if (cls.work && P == 0)
        atomicAdd(cls.work, (unsigned long long)b.n[inst] * (unsigned long long)(b.nsteps[inst] / 2 + 1));
    }
  }

  // Fused solve: the group carries every instance it takes from the queue
  // through contour pass, Anderson step, contour pass, ... until the mixing
  // step reports it finished (converged, non-finite or at the iteration
  // limit), then takes the next one.  No barrier spans more than the group,
  // so instances with short contours or few iterations never wait for the
  // slow ones.
  //
  // Forked paths (m.forks > 0): an instance that takes its update number
  // m.fork_at copies its state into m.forks further paths (mix_step) and
  // publishes them here; groups claim published path jobs in publication order
  // (before each instance of the class queue with m.fork_first, else once the
  // queue is empty) and iterate them the same way.  Groups with nothing to
  // claim wait until every instance of the class has forked or finished
  // (bounded by the time budget and FORK_WAIT_NS of idle waiting); the
  // instances they wait for are all held by running groups, which wait for
  // nothing.
  __device__ static void solve(const BatchDev &b, const ClassDev &cls, const MixDev &m, GroupSmem<R, NW> &S,
                               MixSmem<NW> &MS, int P, int worker, int bar_id) {
    const int lane = P & 31, wid = P >> 5;
    R *slot = reinterpret_cast<R *>(cls.scratch) + (long long)worker * cls.slot_elems;
    auto sync = [&]() { gsync(bar_id); };
    // value of thread 0 for the whole group
    auto bcast = [&](int v) -> int {
      if (NW > 1) {
        if (P == 0) put(S.item, v);
        gsync(bar_id);
        v = S.item;
        gsync(bar_id);
        return v;
      }
      return __shfl_sync(0xffffffffu, v, 0);
    };
    const bool forking = m.forks > 0 && cls.fork_ctl != nullptr;
    auto run_path = [&](int v) {
      const int r = path_of(v, b.base), ii = v - r * b.base;
      // a forked path that can no longer win is not evaluated at all
      if (r > 0 && bcast(P == 0 && fork_key(m, ii, m.iters[v], r) > *(volatile const int *)(m.win + ii))) return;
      for (;;) {
        instance(b, S, P, lane, wid, v, slot, bar_id);
        if (cls.work && P == 0)
          atomicAdd(cls.work, (unsigned long long)b.n[ii] * (unsigned long long)(b.nsteps[ii] / 2 + 1));
        gsync(bar_id);  // density, Q and status of this pass visible to the group
        if (mix_step<NW>(m, v, P, MS, sync)) break;
        if (forking && MS.forked && P == 0) {
          const int k = atomicAdd(cls.fork_ctl, 1);
          atomicExch(cls.fork_list + k, ii + 1);
          __threadfence();
          atomicSub(cls.fork_ctl + 2, 1);
        }
      }
    };
    // Claims the next published path job (thread 0 only): -1 when none is
    // published and unclaimed.  A job is never claimed before its fork is
    // counted; the fork's entry follows its count within a few instructions.
    auto claim = [&]() -> int {
      int h = *(volatile const int *)(cls.fork_ctl + 1);
      for (int tries = 0; tries < 64; tries++) {
        if (h >= *(volatile const int *)cls.fork_ctl * m.forks) return -1;
        const int old = atomicCAS(cls.fork_ctl + 1, h, h + 1);
        if (old == h) {
          const int k = h / m.forks, f = h - k * m.forks;
          int e = 0;
          for (int s = 0; s < (1 << 20) && (e = *(volatile const int *)(cls.fork_list + k)) == 0; s++)
            __nanosleep(100);
          __threadfence();
          return e ? (f + 1) * b.base + (e - 1) : -1;
        }
        h = old;
      }
      return -1;
    };
    for (;;) {
      if (forking && m.fork_first) {
        const int v = bcast(P == 0 ? claim() : -1);
        if (v >= 0) { run_path(v); continue; }
      }
      const int item = bcast(P == 0 ? atomicAdd(cls.head, 1) : 0);
      if (item >= cls.count) break;
      const int inst = cls.items[item];
      if (b.active[inst] == cls.want) run_path(inst);
      // an instance that ends without forking never forks
      if (forking && P == 0 && m.fork_it[inst] == 0) atomicSub(cls.fork_ctl + 2, 1);
    }
    if (!forking) return;
    // the class queue is empty: path jobs until every instance has forked or
    // finished and every published job is claimed
    unsigned long long t0 = (P == 0) ? global_ns() : 0ull;
    for (;;) {
      int v = -1;
      if (P == 0) {
        v = claim();
        if (v < 0) {
          const bool none_left = *(volatile const int *)(cls.fork_ctl + 2) <= 0 &&
                                 *(volatile const int *)(cls.fork_ctl + 1) >= *(volatile const int *)cls.fork_ctl * m.forks;
          const unsigned long long t = global_ns();
          if (none_left || (m.deadline && t > __ldcg(m.deadline)) || t - t0 > FORK_WAIT_NS) v = -2;
          else __nanosleep(4000);
        }
      }
      v = bcast(v);
      if (v == -2) break;
      if (v >= 0) {
        run_path(v);
        if (P == 0) t0 = global_ns();
      }
    }
  }

  // Contour loop of the FP32 increment form on packed pairs (sm_100+ f32x2
  // arithmetic).  Pair i of a thread holds its chunk unknowns i and i + C/2, so
  // the neighbour pairs of pair i are pairs i - 1 and i + 1 except at the two
  // ends, where one lane comes from the neighbouring chunk's shadow value.
  //   * increments are added to the (hi, lo) pair by the fast two-sum
  //     (s = hi + d, lo += d - (s - hi)); every PACKED_RENORM steps the pair is
  //     renormalised (hi = hi + lo, lo = the rounding error of that sum);
  //   * slices of the first half are stored as float2 pairs, [step][pair][thread];
  //   * the density terms are summed in FP32 over blocks of PACKED_BLOCK steps,
  //     and each block sum enters the Kahan-compensated total.
  // The neighbour shadows (qLh/qLl, qRh/qRl) receive the same operations in the
  // same order as the values they mirror, so they stay bit-identical.
  template <typename SepF>
  __device__ static __forceinline__ void contour_f32x2(
      GroupSmem<R, NW> &S, int P, int N, int ns, int half, R *slot, bool last_chunk, R wend,
      const R (&cl)[C], const R (&cd)[C], const R (&cu)[C], const R (&ka)[C], const R (&kb)[C],
      const R (&mm)[CI], const R (&ib)[CI], const R (&ub)[CI], const R (&vc)[CI], const R (&wc)[CI],
      R r_vcn, R r_wcn, SepF &separators, R (&qh)[C], R (&ql)[C], R &qLh, R &qLl, R &qRh, R &qRl,
      R (&acc)[C], R (&cmp)[C]) {
    constexpr int H = C / 2;
    constexpr int kRenorm = PACKED_RENORM, kBlock = PACKED_BLOCK;
    auto sub2 = [](float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); };
    auto mk = [](float a, float b) { return make_float2(a, b); };
    float2 cl2[H], cd2[H], cu2[H], nka2[H], nkb2[H], ib2[H], nvc2[H], nwc2[H];
    float nmm[C], nub[C];
#pragma unroll
    for (int i = 0; i < H; i++) {
      const int u = i + H;  // second node of the pair
      cl2[i] = mk(cl[i], cl[u]);
      cd2[i] = mk(cd[i], cd[u]);
      cu2[i] = mk(cu[i], cu[u]);
      nka2[i] = mk(-ka[i], -ka[u]);
      nkb2[i] = mk(-kb[i], -kb[u]);
      // the separator (node C - 1) has no chunk-interior z: xv = Sp there
      ib2[i] = mk(ib[i], (u < C - 1) ? ib[u < C - 1 ? u : 0] : 0.f);
      nvc2[i] = mk(-vc[i], (u < C - 1) ? -vc[u < C - 1 ? u : 0] : 0.f);
      nwc2[i] = mk(-wc[i], (u < C - 1) ? -wc[u < C - 1 ? u : 0] : 1.f);
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
      nmm[c] = (c >= 1 && c < C - 1) ? -mm[c < C - 1 ? c : 0] : 0.f;
      nub[c] = (c < C - 1) ? -ub[c < C - 1 ? c : 0] : 0.f;
    }
    float2 qh2[H], ql2[H], blk2[H], acc2[H], cmp2[H];
#pragma unroll
    for (int i = 0; i < H; i++) {
      qh2[i] = mk(qh[i], qh[i + H]);
      ql2[i] = mk(0.f, 0.f);
      blk2[i] = acc2[i] = cmp2[i] = mk(0.f, 0.f);
    }
    float2 *slot2 = reinterpret_cast<float2 *>(slot);
    // a pair is stored and read back when its first node is a real unknown
    auto live = [&](int i) { return P * C + i < N; };
#pragma unroll
    for (int i = 0; i < H; i++)
      if (live(i)) slot2[(long long)i * T + P] = qh2[i];

    // one implicit-Euler step: q += D^{-1} (-ds (K + W) q)
    auto step = [&]() {
      float2 r2[H];
      {
        const float2 lh = mk(qLh, qh2[H - 1].x), ll = mk(qLl, ql2[H - 1].x);
        const float2 rh = mk(qh2[0].y, qRh), rl = mk(ql2[0].y, qRl);
#pragma unroll
        for (int i = 0; i < H; i++) {
          const float2 Lh = (i == 0) ? lh : qh2[i > 0 ? i - 1 : 0];
          const float2 Ll = (i == 0) ? ll : ql2[i > 0 ? i - 1 : 0];
          const float2 Rh = (i == H - 1) ? rh : qh2[i < H - 1 ? i + 1 : 0];
          const float2 Rl = (i == H - 1) ? rl : ql2[i < H - 1 ? i + 1 : 0];
          float2 m = __fmul2_rn(cd2[i], qh2[i]);
          m = __ffma2_rn(cl2[i], Lh, m);
          m = __ffma2_rn(cu2[i], Rh, m);
          const float2 d1 = __fadd2_rn(sub2(qh2[i], Lh), sub2(ql2[i], Ll));
          const float2 d2 = __fadd2_rn(sub2(qh2[i], Rh), sub2(ql2[i], Rl));
          r2[i] = __ffma2_rn(nka2[i], d1, __ffma2_rn(nkb2[i], d2, m));
        }
      }
      // chunk-interior Thomas sweep (unknowns 0 .. C-2); y of the separator is 0
      float y[C];
      y[0] = r2[0].x;
#pragma unroll
      for (int c = 1; c < C; c++) {
        const float rc = (c < H) ? r2[c < H ? c : 0].x : r2[c >= H ? c - H : 0].y;
        y[c] = (c < C - 1) ? __fmaf_rn(nmm[c], y[c - 1], rc) : 0.f;
      }
      float2 z2[H];
#pragma unroll
      for (int i = 0; i < H; i++) z2[i] = __fmul2_rn(mk(y[i], y[i + H]), ib2[i]);
      float z[C];
#pragma unroll
      for (int i = 0; i < H; i++) { z[i] = z2[i].x; z[i + H] = z2[i].y; }
#pragma unroll
      for (int c = C - 3; c >= 0; c--) z[c] = __fmaf_rn(nub[c], z[c + 1], z[c]);
#pragma unroll
      for (int i = 0; i < H; i++) z2[i] = mk(z[i], z[i + H]);
      const float rlast = r2[H - 1].y;
      float zc0n, Sp, Sprev, Snext;
      separators(z[0], z[C - 2], rlast, zc0n, Sp, Sprev, Snext);
      const float2 Sp2 = mk(Sp, Sp), Sq2 = mk(Sprev, Sprev);
      const float dL = Sprev;
      const float dR = last_chunk ? 0.f : __fmaf_rn(-r_wcn, Snext, __fmaf_rn(-r_vcn, Sp, zc0n));
#pragma unroll
      for (int i = 0; i < H; i++) {
        const float2 xv = __ffma2_rn(nwc2[i], Sp2, __ffma2_rn(nvc2[i], Sq2, z2[i]));
        const float2 sum = __fadd2_rn(qh2[i], xv);
        ql2[i] = __fadd2_rn(ql2[i], sub2(xv, sub2(sum, qh2[i])));
        qh2[i] = sum;
      }
      {
        const float s1 = __fadd_rn(qLh, dL);
        qLl = __fadd_rn(qLl, __fsub_rn(dL, __fsub_rn(s1, qLh)));
        qLh = s1;
        const float s2 = __fadd_rn(qRh, dR);
        qRl = __fadd_rn(qRl, __fsub_rn(dR, __fsub_rn(s2, qRh)));
        qRh = s2;
      }
    };
    auto renorm = [&]() {
#pragma unroll
      for (int i = 0; i < H; i++) {
        const float2 h = __fadd2_rn(qh2[i], ql2[i]);
        ql2[i] = sub2(ql2[i], sub2(h, qh2[i]));
        qh2[i] = h;
      }
      float h = __fadd_rn(qLh, qLl);
      qLl = __fsub_rn(qLl, __fsub_rn(h, qLh));
      qLh = h;
      h = __fadd_rn(qRh, qRl);
      qRl = __fsub_rn(qRl, __fsub_rn(h, qRh));
      qRh = h;
    };
    auto flush = [&]() {
#pragma unroll
      for (int i = 0; i < H; i++) {
        const float2 yv = sub2(blk2[i], cmp2[i]);
        const float2 tt = __fadd2_rn(acc2[i], yv);
        cmp2[i] = sub2(sub2(tt, acc2[i]), yv);
        acc2[i] = tt;
        blk2[i] = mk(0.f, 0.f);
      }
    };
    auto weight = [&](int k) { return (k == ns) ? wend : S.qw[min(__ffs(k) - 1, 14)]; };

    // first half: store slices 1..half (the middle slice pairs with itself when ns is even)
    for (int k = 1; k <= half; k++) {
      step();
      if ((k & (kRenorm - 1)) == 0) renorm();
      float2 *dst = slot2 + (long long)k * H * T + P;
#pragma unroll
      for (int i = 0; i < H; i++)
        if (live(i)) dst[(long long)i * T] = qh2[i];
      if (k == ns - k) {
        const float wk = weight(k);
#pragma unroll
        for (int i = 0; i < H; i++) blk2[i] = __ffma2_rn(__fmul2_rn(mk(wk, wk), qh2[i]), qh2[i], blk2[i]);
      }
    }
    // second half: slice k pairs with the stored slice ns - k (prefetched one step ahead)
    float2 nxt2[H];
    {
      const float2 *src = slot2 + (long long)(ns - half - 1) * H * T + P;
#pragma unroll
      for (int i = 0; i < H; i++) nxt2[i] = live(i) ? src[(long long)i * T] : mk(0.f, 0.f);
    }
    int nblk = 0;
    for (int k = half + 1; k <= ns; k++) {
      float2 pre2[H];
#pragma unroll
      for (int i = 0; i < H; i++) pre2[i] = nxt2[i];
      if (CL == 1 && k + PREFETCH_STEPS < ns) {
        const float2 *pf = slot2 + (long long)(ns - k - 1 - PREFETCH_STEPS) * H * T + P;
#pragma unroll
        for (int i = 0; i < H; i++)
          if (live(i)) prefetch_l2(pf + (long long)i * T);
      }
      if (k < ns) {
        const float2 *src = slot2 + (long long)(ns - k - 1) * H * T + P;
#pragma unroll
        for (int i = 0; i < H; i++) nxt2[i] = live(i) ? src[(long long)i * T] : mk(0.f, 0.f);
      }
      step();
      if ((k & (kRenorm - 1)) == 0) renorm();
      const float w2 = 2.f * weight(k);
#pragma unroll
      for (int i = 0; i < H; i++) blk2[i] = __ffma2_rn(__fmul2_rn(mk(w2, w2), qh2[i]), pre2[i], blk2[i]);
      if (++nblk == kBlock) { flush(); nblk = 0; }
    }
    flush();
#pragma unroll
    for (int i = 0; i < H; i++) {
      qh[i] = qh2[i].x; qh[i + H] = qh2[i].y;
      ql[i] = ql2[i].x; ql[i + H] = ql2[i].y;
      acc[i] = acc2[i].x; acc[i + H] = acc2[i].y;
      cmp[i] = cmp2[i].x; cmp[i + H] = cmp2[i].y;
    }
  }

  __device__ static void instance(const BatchDev &b, GroupSmem<R, NW> &S, int P, int lane, int wid,
                                  int inst, R *slot, int bar_id) {
    const unsigned FULL = 0xffffffffu;
    const int path = path_of(inst, b.base), ii = inst - path * b.base;  // forked path and instance
    const int n = b.n[ii], N = n - 2, ns = b.nsteps[ii], half = ns / 2;
    const double ds = b.ds[ii];
    const long long off = b.node_off[ii], doff = off + path * b.rep_nodes;
    const double *x = b.x + off;
    const double *w = b.w + doff;
    {
      const int loc = (CL > 1) ? (int)threadIdx.x : P;  // every CTA of a cluster keeps its own weights
      if (loc < 16) S.qw[loc] = (R)b.qw[(long long)ii * 16 + loc];
    }
    gsync(bar_id);
    int bad = 0;

    // ---------------- setup (FP64): bands, chunk LU, spikes ----------------
    // Right-hand side bands.  Direct form: the mass matrix.  Increment form:
    // -ds (K + W) q with the stiffness applied to node differences (ka, kb =
    // ds/a1, ds/a2) so that it vanishes exactly on constants in FP32, and the
    // field term -ds w M in (cl, cd, cu).
    double dl[C], dd[C], du[C];
    R cl[C], cd[C], cu[C], ka[C], kb[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
      const int j = P * C + c;
      ka[c] = kb[c] = (R)0;
      if (j < N) {
        const int i = j + 1;
        const double a1 = x[i] - x[i - 1], a2 = x[i + 1] - x[i];
        const double ml = a1 / 6.0, md = a1 / 3.0 + a2 / 3.0, mu = a2 / 6.0;
        const double kl = -1.0 / a1, kd = 1.0 / a1 + 1.0 / a2, ku = -1.0 / a2;
        const double wi = __ldcg(w + i);  // L2: the fused solve updates w between passes
        const double al = kl + wi * ml, ad = kd + wi * md, au = ku + wi * mu;
        dl[c] = (j == 0) ? 0.0 : ml + ds * al;
        dd[c] = md + ds * ad;
        du[c] = (j == N - 1) ? 0.0 : mu + ds * au;
        if constexpr (DELTA) {
          ka[c] = (R)(ds / a1);
          kb[c] = (R)(ds / a2);
          cl[c] = (R)((j == 0) ? 0.0 : -ds * wi * ml);
          cd[c] = (R)(-ds * wi * md);
          cu[c] = (R)((j == N - 1) ? 0.0 : -ds * wi * mu);
        } else {
          cl[c] = (R)((j == 0) ? 0.0 : ml);
          cd[c] = (R)md;
          cu[c] = (R)((j == N - 1) ? 0.0 : mu);
        }
        if (!(dd[c] > fabs(dl[c]) + fabs(du[c]))) bad |= ST_NOT_DOMINANT;
      } else {
        dl[c] = 0.0; dd[c] = 1.0; du[c] = 0.0;
        cl[c] = cd[c] = cu[c] = (R)0;
      }
    }
    // chunk-interior LU (unknowns 0..C-2) and spikes
    R mm[CI], ib[CI], ub[CI], vc[CI], wc[CI];
    double vc0 = 0.0, wc0 = 0.0, vcl = 0.0, wcl = 0.0;  // spikes at interior index 0 and C-2
    if (C > 1) {
      double ibd[CI], ubd[CI], mmd[CI], v[CI], ww[CI];
      double beta = dd[0];
      ibd[0] = 1.0 / beta; ubd[0] = du[0] * ibd[0]; mmd[0] = 0.0;
#pragma unroll
      for (int k = 1; k < C - 1; k++) {
        mmd[k] = dl[k] * ibd[k - 1];
        beta = dd[k] - mmd[k] * du[k - 1];
        ibd[k] = 1.0 / beta;
        ubd[k] = du[k] * ibd[k];
      }
      // v = D_II^{-1} (dl[0] e_0),  w = D_II^{-1} (du[C-2] e_{C-2})
      v[0] = dl[0];
#pragma unroll
      for (int k = 1; k < C - 1; k++) v[k] = -mmd[k] * v[k - 1];
      v[C - 2] *= ibd[C - 2];
#pragma unroll
      for (int k = C - 3; k >= 0; k--) v[k] = v[k] * ibd[k] - ubd[k] * v[k + 1];
      ww[C - 2] = du[C - 2] * ibd[C - 2];
#pragma unroll
      for (int k = C - 3; k >= 0; k--) ww[k] = -ubd[k] * ww[k + 1];
#pragma unroll
      for (int k = 0; k < C - 1; k++) {
        mm[k] = (R)mmd[k]; ib[k] = (R)ibd[k]; ub[k] = (R)ubd[k];
        vc[k] = (R)v[k]; wc[k] = (R)ww[k];
      }
      vc0 = v[0]; wc0 = ww[0]; vcl = v[C - 2]; wcl = ww[C - 2];
    } else {
#pragma unroll
      for (int k = 0; k < CI; k++) mm[k] = ib[k] = ub[k] = vc[k] = wc[k] = (R)0;
    }
    // next chunk's spikes at its first interior unknown (lane 31: from the next warp)
    double vcn = __shfl_down_sync(FULL, vc0, 1), wcn = __shfl_down_sync(FULL, wc0, 1);
    if (NW > 1) {
      if (lane == 0) { put(S.s_vc0[wid], vc0); put(S.s_wc0[wid], wc0); }
      gsync(bar_id);
      if (lane == 31) {
        vcn = (wid + 1 < NW) ? S.s_vc0[wid + 1] : 0.0;
        wcn = (wid + 1 < NW) ? S.s_wc0[wid + 1] : 0.0;
      }
    } else if (lane == 31) {
      vcn = 0.0; wcn = 0.0;
    }
    // chunk-separator system: al_p S_{p-1} + be_p S_p + ga_p S_{p+1} = rho_p
    const double dls = dl[C - 1], dds = dd[C - 1], dus = du[C - 1];
    double al, be, ga;
    if (C > 1) {
      al = -dls * vcl;
      be = dds - dls * wcl - dus * vcn;
      ga = -dus * wcn;
    } else {
      al = dls; be = dds; ga = dus;
    }
    // warp level: lanes 0..30 interior (couplings of lane 0 to the previous warp
    // separator and of lane 30 to lane 31 moved into spikes), lane 31 identity
    R K1[5], K2[5];
    R ibw;
    double vw, ww;
    {
      // NW == 1: the 32 chunk separators form one self-contained system (no
      // coupling outside the warp), solved directly by PCR over all lanes.
      double a = (lane == 0 || (NW > 1 && lane == 31)) ? 0.0 : al;
      double bb = (NW > 1 && lane == 31) ? 1.0 : be;
      double c = (NW > 1 ? lane >= 30 : lane == 31) ? 0.0 : ga;
      double k1d[5], k2d[5];
#pragma unroll
      for (int l = 0; l < 5; l++) {
        const int s = 1 << l;
        const double am = __shfl_up_sync(FULL, a, s), bm = __shfl_up_sync(FULL, bb, s),
                     cm = __shfl_up_sync(FULL, c, s);
        const double ap = __shfl_down_sync(FULL, a, s), bp = __shfl_down_sync(FULL, bb, s),
                     cp = __shfl_down_sync(FULL, c, s);
        const double k1 = (lane >= s) ? a / bm : 0.0;
        const double k2 = (lane + s < 32) ? c / bp : 0.0;
        const double na = -k1 * am, nc = -k2 * cp, nb = bb - k1 * cm - k2 * ap;
        a = na; c = nc; bb = nb;
        k1d[l] = k1; k2d[l] = k2;
        K1[l] = (R)k1; K2[l] = (R)k2;
      }
      const double ibwd = 1.0 / bb;
      ibw = (R)ibwd;
      // spikes of the warp interior system
      double rv = (lane == 0) ? al : 0.0, rw = (lane == 30) ? ga : 0.0;
#pragma unroll
      for (int l = 0; l < 5; l++) {
        const int s = 1 << l;
        const double vm = __shfl_up_sync(FULL, rv, s), vp = __shfl_down_sync(FULL, rv, s);
        const double wm = __shfl_up_sync(FULL, rw, s), wp = __shfl_down_sync(FULL, rw, s);
        rv = rv - k1d[l] * vm - k2d[l] * vp;
        rw = rw - k1d[l] * wm - k2d[l] * wp;
      }
      vw = (NW == 1 || lane == 31) ? 0.0 : rv * ibwd;
      ww = (NW == 1 || lane == 31) ? 0.0 : rw * ibwd;
    }
    // level 2: warp separators
    const double vw30 = __shfl_sync(FULL, vw, 30), ww30 = __shfl_sync(FULL, ww, 30);
    double vwn = 0.0, wwn = 0.0;
    R K1b[L2 > 0 ? L2 : 1], K2b[L2 > 0 ? L2 : 1];
    R iB2;
    if (NW > 1) {
      if (lane == 0) { put(S.s_vw0[wid], vw); put(S.s_ww0[wid], ww); }
      gsync(bar_id);
      if (lane == 31) {
        vwn = (wid + 1 < NW) ? S.s_vw0[wid + 1] : 0.0;
        wwn = (wid + 1 < NW) ? S.s_ww0[wid + 1] : 0.0;
        put(S.s_A[wid], (wid == 0) ? 0.0 : -al * vw30);
        put(S.s_B[wid], be - al * ww30 - ga * vwn);
        put(S.s_C[wid], (wid + 1 < NW) ? -ga * wwn : 0.0);
      }
      gsync(bar_id);
      double a = (lane < NW) ? S.s_A[lane] : 0.0;
      double bb = (lane < NW) ? S.s_B[lane] : 1.0;
      double c = (lane < NW) ? S.s_C[lane] : 0.0;
#pragma unroll
      for (int l = 0; l < L2; l++) {
        const int s = 1 << l;
        const double am = __shfl_up_sync(FULL, a, s), bm = __shfl_up_sync(FULL, bb, s),
                     cm = __shfl_up_sync(FULL, c, s);
        const double ap = __shfl_down_sync(FULL, a, s), bp = __shfl_down_sync(FULL, bb, s),
                     cp = __shfl_down_sync(FULL, c, s);
        const double k1 = (lane >= s) ? a / bm : 0.0;
        const double k2 = (lane + s < NW) ? c / bp : 0.0;
        const double na = -k1 * am, nc = -k2 * cp, nb = bb - k1 * cm - k2 * ap;
        a = na; c = nc; bb = nb;
        K1b[l] = (R)k1; K2b[l] = (R)k2;
      }
      iB2 = (R)(1.0 / bb);
    } else {
      K1b[0] = K2b[0] = (R)0;
      iB2 = (R)(1.0 / (be - al * ww30));  // meaningful in lane 31
    }
    const R r_al = (R)al, r_ga = (R)ga, r_vw = (R)vw, r_ww = (R)ww, r_vwn = (R)vwn, r_wwn = (R)wwn;
    const R r_dls = (R)dls, r_dus = (R)dus, r_vcn = (R)vcn, r_wcn = (R)wcn;
    const bool last_chunk = (P == T - 1);

    // Cluster classes: the exchange steps taken so far, whether the exchange
    // failed, and lane l's coefficients of warp l's right-hand side on warp
    // l+1's values (C == 1: no zc0 term).
    unsigned xk = 0;
    bool xbad = false;
    R xdus = (R)0, xga = (R)0;
    if constexpr (CL > 1) {
      xk = S.xk;
      xbad = S.xfail != 0;
      if (lane == 31) { put(S.c_dus[wid], (C > 1) ? r_dus : (R)0); put(S.c_ga[wid], r_ga); }
      gsync(bar_id);
      if (lane < NW) { xdus = S.c_dus[lane]; xga = S.c_ga[lane]; }
    }
    // Bounded wait for phase `parity` of one of this CTA's exchange mbarriers.
    auto xwait = [&](unsigned bar, unsigned parity) {
      if (xbad || cx_test(bar, parity)) return;
      const unsigned long long t0 = global_ns();
      for (;;) {
        if (*(volatile int *)&S.xfail) { xbad = true; return; }
        if (cx_test(bar, parity)) return;
        if (global_ns() - t0 > CX_WAIT_NS) {
          xbad = true;
          for (int r = 0; r < CL; r++)
            asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cx_remote(cx_smem(&S.xfail), r)), "r"(1)
                         : "memory");
          return;
        }
      }
    };

    // Separator solve of one contour step.  In: this thread's chunk-local z at
    // its first and last interior unknowns and the right-hand side at its
    // separator (C == 1: the right-hand side).  Out: the next chunk's z at its
    // first unknown, this thread's separator value and its neighbours'.
    auto separators = [&](R zc0, R zcl, R rl, R &zc0n, R &Sp, R &Sprev, R &Snext) {
      zc0n = __shfl_down_sync(FULL, zc0, 1);
      // chunk-separator right-hand side and warp-interior PCR
      R rho = (C > 1) ? fmaR(-r_dus, zc0n, fmaR(-r_dls, zcl, rl)) : rl;
      R t = (NW == 1 || lane != 31) ? rho : (R)0;
#pragma unroll
      for (int l = 0; l < 5; l++) {
        const int s = 1 << l;
        const R tm = __shfl_up_sync(FULL, t, s), tp = __shfl_down_sync(FULL, t, s);
        t = fmaR(-K2[l], tp, fmaR(-K1[l], tm, t));
      }
      if constexpr (NW == 1) {
        Sp = t * ibw;
        Sprev = __shfl_up_sync(FULL, Sp, 1);
        Snext = __shfl_down_sync(FULL, Sp, 1);
        if (lane == 0) Sprev = (R)0;
        if (lane == 31) Snext = (R)0;
      } else {
        const R zw = t * ibw;
        const R zw30 = __shfl_sync(FULL, zw, 30);
        R zwn = (R)0;
        R t2;
        if constexpr (CL > 1) {
          const unsigned par = xk & 1u;
          if (!xbad) {
            if (lane == 0) {
#pragma unroll
              for (int r = 0; r < CL; r++) {
                const unsigned rb = cx_remote(cx_smem(&S.xbar[par]), r);
                cx_send(cx_remote(cx_smem(&S.x_Z0[par][wid]), r), zc0, rb);
                cx_send(cx_remote(cx_smem(&S.x_ZW[par][wid]), r), zw, rb);
              }
            } else if (lane == 31) {
              const R A = fmaR(-r_al, zw30, (C > 1) ? fmaR(-r_dls, zcl, rl) : rl);
#pragma unroll
              for (int r = 0; r < CL; r++)
                cx_send(cx_remote(cx_smem(&S.x_A[par][wid]), r), A, cx_remote(cx_smem(&S.xbar[par]), r));
            }
          }
          xwait(cx_smem(&S.xbar[par]), (xk >> 1) & 1u);
          if (threadIdx.x == 0 && !xbad) cx_arm(cx_smem(&S.xbar[par]), 3 * NW * sizeof(R));
          // lane l < NW: warp l's right-hand side (the last warp has no next)
          const int ln = min(lane + 1, NW - 1), la = min(lane, NW - 1);
          const bool nx = lane + 1 < NW;
          const R z0n = nx ? S.x_Z0[par][ln] : (R)0, zwl = nx ? S.x_ZW[par][ln] : (R)0;
          const R rA = S.x_A[par][la];
          t2 = (lane < NW) ? fmaR(-xga, zwl, fmaR(-xdus, z0n, rA)) : (R)0;
          if (lane == 31) {  // the next warp's first-lane values (zero after the last warp)
            const int wn = min(wid + 1, NW - 1);
            const bool hn = wid + 1 < NW;
            const R zcx = hn ? S.x_Z0[par][wn] : (R)0;
            zwn = hn ? S.x_ZW[par][wn] : (R)0;
            if (C > 1) zc0n = zcx;
          }
          xk++;
        } else {
          if (lane == 0) { put(S.pub_zc0[wid], zc0); put(S.pub_zw[wid], zw); }
          gsync(bar_id);
          if (lane == 31) {
            const bool has_next = (wid + 1 < NW);
            const R zcx = has_next ? S.pub_zc0[wid + 1] : (R)0;
            zwn = has_next ? S.pub_zw[wid + 1] : (R)0;
            if (C > 1) {
              zc0n = zcx;
              rho = fmaR(-r_dus, zcx, fmaR(-r_dls, zcl, rl));
            }
            put(S.pub_R[wid], fmaR(-r_ga, zwn, fmaR(-r_al, zw30, rho)));
          }
          gsync(bar_id);
          t2 = (lane < NW) ? S.pub_R[lane] : (R)0;
        }
#pragma unroll
        for (int l = 0; l < L2; l++) {
          const int s = 1 << l;
          const R tm = __shfl_up_sync(FULL, t2, s), tp = __shfl_down_sync(FULL, t2, s);
          t2 = fmaR(-K2b[l], tp, fmaR(-K1b[l], tm, t2));
        }
        const R sw = t2 * iB2;
        const R Sown = __shfl_sync(FULL, sw, wid);
        R Sprevw = __shfl_sync(FULL, sw, wid > 0 ? wid - 1 : 0);
        R Snextw = __shfl_sync(FULL, sw, wid + 1 < NW ? wid + 1 : wid);
        if (wid == 0) Sprevw = (R)0;
        if (wid + 1 >= NW) Snextw = (R)0;
        // separator values and their neighbours
        Sp = (lane == 31) ? Sown : fmaR(-r_ww, Sown, fmaR(-r_vw, Sprevw, zw));
        Sprev = __shfl_up_sync(FULL, Sp, 1);
        Snext = __shfl_down_sync(FULL, Sp, 1);
        if (lane == 0) Sprev = Sprevw;
        if (lane == 31) Snext = (wid + 1 < NW) ? fmaR(-r_wwn, Snextw, fmaR(-r_vwn, Sown, zwn)) : (R)0;
      }
    };

    // ---------------- state ----------------
    R qh[C], ql[C], acc[C], cmp[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
      const int j = P * C + c;
      qh[c] = (j < N) ? (R)1 : (R)0;
      ql[c] = (R)0; acc[c] = (R)0; cmp[c] = (R)0;
    }
    R qLh = (P * C - 1 >= 0 && P * C - 1 < N) ? (R)1 : (R)0, qLl = (R)0;
    R qRh = ((P + 1) * C < N) ? (R)1 : (R)0, qRl = (R)0;
    const R wend = S.qw[15];
    if constexpr (DELTA && C >= 2 && std::is_same<R, float>::value) {
      contour_f32x2(S, P, N, ns, half, slot, last_chunk, wend, cl, cd, cu, ka, kb, mm, ib, ub, vc, wc,
                    r_vcn, r_wcn, separators, qh, ql, qLh, qLl, qRh, qRl, acc, cmp);
    } else {
    // padded unknowns (P*C + c >= N) are never stored or read back
#pragma unroll
    for (int c = 0; c < C; c++)
      if (P * C + c < N) slot[(long long)c * T + P] = qh[c];

    // ---------------- contour loop ----------------
    // The slice read back at step k (ns - k) is prefetched during step k-1
    // when it was stored before step k-1; otherwise it is loaded in step k.
    R nxt[C];
    bool have_nxt = false;
    for (int k = 1; k <= ns; k++) {
      const bool acc_step = (k >= ns - half);
      const bool self_pair = (k == ns - k);
      R pre[C];
      if (acc_step && !self_pair) {
        if (have_nxt) {
#pragma unroll
          for (int c = 0; c < C; c++) pre[c] = nxt[c];
        } else {
          const R *src = slot + (long long)(ns - k) * TC + P;
#pragma unroll
          for (int c = 0; c < C; c++) pre[c] = (P * C + c < N) ? src[(long long)c * T] : (R)0;
        }
      }
      // prefetch for step k+1: its slice ns-k-1 must have been stored at a step < k
      have_nxt = (k + 1 <= ns) && (k + 1 >= ns - half) && (k + 1 != ns - k - 1) && (ns - k - 1 < k);
      if (have_nxt) {
        const R *src = slot + (long long)(ns - k - 1) * TC + P;
#pragma unroll
        for (int c = 0; c < C; c++) nxt[c] = (P * C + c < N) ? src[(long long)c * T] : (R)0;
      }
      // right-hand side
      R r[C];
#pragma unroll
      for (int c = 0; c < C; c++) {
        const R left = (c == 0) ? qLh : qh[c - 1];
        const R right = (c == C - 1) ? qRh : qh[c + 1];
        r[c] = fmaR(cu[c], right, fmaR(cl[c], left, cd[c] * qh[c]));
        if constexpr (DELTA) {
          const R leftl = (c == 0) ? qLl : ql[c - 1];
          const R rightl = (c == C - 1) ? qRl : ql[c + 1];
          const R d1 = (qh[c] - left) + (ql[c] - leftl);
          const R d2 = (qh[c] - right) + (ql[c] - rightl);
          r[c] -= fmaR(ka[c], d1, kb[c] * d2);
        }
      }
      // chunk-interior Thomas sweep
      R zc[CI];
      if (C > 1) {
        R y = r[0];
        zc[0] = y;
#pragma unroll
        for (int kk = 1; kk < C - 1; kk++) { y = fmaR(-mm[kk], y, r[kk]); zc[kk] = y; }
        zc[C - 2] = zc[C - 2] * ib[C - 2];
#pragma unroll
        for (int kk = C - 3; kk >= 0; kk--) zc[kk] = fmaR(-ub[kk], zc[kk + 1], zc[kk] * ib[kk]);
      } else {
        zc[0] = (R)0;
      }
      R zc0n, Sp, Sprev, Snext;
      separators(zc[0], zc[C > 1 ? C - 2 : 0], (C > 1) ? r[C - 1] : r[0], zc0n, Sp, Sprev, Snext);
      // chunk unknowns
      R xv[C];
#pragma unroll
      for (int c = 0; c < C - 1; c++) xv[c] = fmaR(-wc[c], Sp, fmaR(-vc[c], Sprev, zc[c]));
      xv[C - 1] = Sp;
      const R dL = Sprev;
      R dR = (C > 1) ? fmaR(-r_wcn, Snext, fmaR(-r_vcn, Sp, zc0n)) : Snext;
      if (last_chunk) dR = (R)0;
      if constexpr (DELTA) {
#pragma unroll
        for (int c = 0; c < C; c++) ff_add(qh[c], ql[c], xv[c]);
        ff_add(qLh, qLl, dL);
        ff_add(qRh, qRl, dR);
      } else {
#pragma unroll
        for (int c = 0; c < C; c++) qh[c] = xv[c];
        qLh = dL;
        qRh = dR;
      }
      // half-contour store / density accumulation
      if (k <= half) {
        R *dst = slot + (long long)k * TC + P;
#pragma unroll
        for (int c = 0; c < C; c++)
          if (P * C + c < N) dst[(long long)c * T] = qh[c];
      }
      if (acc_step) {
        R wk = (k == ns) ? wend : S.qw[min(__ffs(k) - 1, 14)];
        if (!self_pair) wk = wk + wk;
#pragma unroll
        for (int c = 0; c < C; c++) {
          const R other = self_pair ? qh[c] : pre[c];
          const R term = (wk * qh[c]) * other;
          if constexpr (DELTA) {
            const R y = term - cmp[c];
            const R tt = acc[c] + y;
            cmp[c] = (tt - acc[c]) - y;
            acc[c] = tt;
          } else {
            acc[c] += term;
          }
        }
      }
    }

    }  // contour loop of the direct form / C == 1

    // ---------------- epilogue: phi, Q, status ----------------
    double qpart = 0.0;
    double *phi = b.phi + doff;
#pragma unroll
    for (int c = 0; c < C; c++) {
      const int j = P * C + c;
      if (j < N) {
        const double v = (double)acc[c] - (double)cmp[c];
        if (!isfinite(v)) bad |= ST_NONFINITE;
        phi[j + 1] = v;
        qpart += 0.5 * (x[j + 2] - x[j]) * ((double)qh[c] + (double)ql[c]);
      }
    }
    if (P == 0) { phi[0] = 0.0; phi[n - 1] = 0.0; }
    if constexpr (CL > 1) {
      if (xbad) bad |= ST_WATCHDOG;  // an exchange wait ran out: this pass is void
      if (threadIdx.x == 0) S.xk = xk;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      qpart += __shfl_down_sync(FULL, qpart, s);
      bad |= __shfl_down_sync(FULL, bad, s);
    }
    if (NW > 1) {
      if (lane == 0) { put(S.red[wid], qpart); put(S.ired[wid], bad); }
      gsync(bar_id);
      if (P == 0) {
        qpart = 0.0;
        for (int q = 0; q < NW; q++) { qpart += S.red[q]; bad |= S.ired[q]; }
      }
      gsync(bar_id);
    }
    if (P == 0) {
      b.Q[inst] = qpart / (x[n - 1] - x[0]);
      if (bad) atomicOr(&b.status[inst], bad);
    }
  }
};

template <typename R, int C, int NW, bool DELTA>
__global__ void __launch_bounds__(Propagator<R, C, NW, DELTA>::CTA, 1)
propagate_kernel(BatchDev b, ClassDev cls) {
  using Pp = Propagator<R, C, NW, DELTA>;
  __shared__ GroupSmem<R, NW> sm[Pp::GPC];
  const int g = threadIdx.x / Pp::T;
  const int P = threadIdx.x % Pp::T;
  const int worker = blockIdx.x * Pp::GPC + g;
  if (worker >= cls.workers) return;
  Pp::run(b, cls, sm[g], P, worker, 1 + g);
}

// Propagator of one large shape class on thread-block clusters of CL CTAs (one
// group per cluster; launched with the cluster dimension as a launch attribute).
template <typename R, int C, int NW, bool DELTA, int CL>
__global__ void __launch_bounds__(32 * NW / CL, 1) propagate_cluster_kernel(BatchDev b, ClassDev cls) {
  using Pp = Propagator<R, C, NW, DELTA, CL>;
  __shared__ GroupSmem<R, NW> sm;
  const int rank = (int)cooperative_groups::this_cluster().block_rank();
  const int P = rank * Pp::CTA + (int)threadIdx.x;
  const int worker = (int)(blockIdx.x / CL);
  if (worker >= cls.workers) return;  // the same for every CTA of the cluster
  if (threadIdx.x == 0) {
    sm.xk = 0;
    sm.xfail = 0;
    for (int i = 0; i < 2; i++) cx_init(cx_smem(&sm.xbar[i]));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // first phase of each step parity: every warp's A, zc0 and zw
    for (int i = 0; i < 2; i++) cx_arm(cx_smem(&sm.xbar[i]), 3 * NW * sizeof(R));
  }
  cooperative_groups::this_cluster().sync();  // barriers initialised before any remote store
  Pp::run(b, cls, sm, P, worker, 1);
}

// Fused persistent solve of one shape class (see Propagator::solve).
template <typename R, int C, int NW, bool DELTA>
__global__ void __launch_bounds__(Propagator<R, C, NW, DELTA>::CTA,
                                  Propagator<R, C, NW, DELTA>::CTA * SOLVE_MIN_CTAS <= 1024 ? SOLVE_MIN_CTAS : 1)
solve_kernel(BatchDev b, ClassDev cls, MixDev m) {
  using Pp = Propagator<R, C, NW, DELTA>;
  __shared__ GroupSmem<R, NW> sm[Pp::GPC];
  __shared__ MixSmem<NW> ms[Pp::GPC];
  const int g = threadIdx.x / Pp::T;
  const int P = threadIdx.x % Pp::T;
  const int worker = blockIdx.x * Pp::GPC + g;
  if (worker >= cls.workers) return;
  Pp::solve(b, cls, m, sm[g], ms[g], P, worker, 1 + g);
}

}  // namespace scft
