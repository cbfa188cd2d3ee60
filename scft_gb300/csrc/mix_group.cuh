// mix_group.cuh -- one batched Anderson iteration of one instance, carried out
// by a group of 32*NW threads (FP64).  Used by the one-CTA-per-instance
// mix_kernel (NW = 8, __syncthreads) and by the fused solve kernels, where the
// propagator's own group runs the update between two contour passes (named
// barrier).
//
// The step: residual check, difference-form history of the mixing residual,
// weighted regularised least squares, a preconditioned and clipped step,
// restart safeguard (the safeguarded form of adm.c:24-313 / ADM_chen_C.c:18-147
// used by the batched solver; the CPU restatement is or_anderson_solve in the
// oracle).
#pragma once
#include "mixing.cuh"

namespace scft {

constexpr int MIX_MAXD = 16;

__device__ __forceinline__ double warp_max(double v) {
  for (int s = 16; s > 0; s >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, s));
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  return v;
}

// Solve the k x k system A g = b (row-major, A overwritten) by Gaussian
// elimination with partial pivoting; single thread.
__device__ inline void small_solve(double *A, double *b, int k) {
  for (int c = 0; c < k; c++) {
    int p = c;
    double big = fabs(A[c * k + c]);
    for (int r = c + 1; r < k; r++)
      if (fabs(A[r * k + c]) > big) { big = fabs(A[r * k + c]); p = r; }
    if (p != c) {
      for (int j = 0; j < k; j++) { double t = A[c * k + j]; A[c * k + j] = A[p * k + j]; A[p * k + j] = t; }
      double t = b[c]; b[c] = b[p]; b[p] = t;
    }
    double piv = A[c * k + c];
    if (piv == 0.0) piv = 1e-300;
    for (int r = c + 1; r < k; r++) {
      double f = A[r * k + c] / piv;
      for (int j = c; j < k; j++) A[r * k + j] -= f * A[c * k + j];
      b[r] -= f * b[c];
    }
  }
  for (int c = k - 1; c >= 0; c--) {
    double s = b[c];
    for (int j = c + 1; j < k; j++) s -= A[c * k + j] * b[j];
    double piv = A[c * k + c];
    b[c] = s / (piv == 0.0 ? 1e-300 : piv);
  }
}

// Shared memory of one group's mixing step.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <int NW>
struct MixSmem {
  double sm[NW];
  double red[2 * MIX_MAXD][NW];
  double gam[MIX_MAXD];
  int slot[MIX_MAXD];
  int ctl[4];
  int stop;
  int forked;   // set by mix_step when this update copied the instance into its forked paths
};

// Group-wide max of v (every thread of the group receives it).
template <int NW, typename Sync>
__device__ __forceinline__ double group_max(double v, MixSmem<NW> &S, int tid, Sync &sync) {
  const int lane = tid & 31, wid = tid >> 5;
  v = warp_max(v);
  sync();
  if (lane == 0) S.sm[wid] = v;
  sync();
  double r = (lane < NW) ? S.sm[lane] : 0.0;
  return warp_max(r);
}

// Key of path r of instance ii converging after `it` updates (see
// MixDev::win): the instance's own path (r = 0) before its fork or within the
// grace updates after it beats every path.
__device__ __forceinline__ int fork_key(const MixDev &m, int ii, int it, int r) {
  if (r == 0) {
    const int fit = m.fork_it[ii];
    if (fit == 0 || it <= fit + m.fork_grace) return 0;
  }
  return it * 16 + r;
}

// One Anderson iteration of instance `inst` by threads tid = 0 .. 32*NW-1 of a
// group; `sync` is the group's barrier.  Returns true (in every thread) when the
// instance is finished: converged (or handed to the FP64 check), non-finite, or
// at the iteration limit.  On false the field m.w of the instance holds the next
// iterate.
template <int NW, typename Sync>
__device__ bool mix_step(const MixDev &m, int inst, int tid, MixSmem<NW> &S, Sync &sync) {
  constexpr int NT = 32 * NW;
  const int lane = tid & 31, wid = tid >> 5;
  const int act = m.active[inst];
  const int r = path_of(inst, m.base), ii = inst - r * m.base;  // path and instance
  const int n = m.n[ii], N = n - 2;
  const long long no = m.node_off[ii], io = m.int_off[ii];
  const long long dno = no + r * m.rep_nodes, dio = io + r * m.rep_int;
  const double *x = m.x + no, *f0 = m.f0 + no, *phi = m.phi + dno;
  double *w = m.w + dno;
  double *graw = m.graw + dio, *gcur = m.gcur + dio, *gprev = m.gprev + dio, *wprev = m.wprev + dio;
  const int D = m.depth;
  double *hdx = m.hdx + dio * D, *hdg = m.hdg + dio * D;
  double *G = m.gram + (long long)inst * D * D;

  // 1. residual, its norm, raw mixing residual
  double e = 0.0, badv = 0.0;
  for (int j = tid; j < N; j += NT) {
    // L2 loads: in the fused solve phi was written by other threads of this kernel
    const double p = __ldcg(phi + j + 1), f = f0[j + 1], r = p - f;
    if (!isfinite(r)) badv = 1.0;
    e = fmax(e, fabs(r));
    graw[j] = m.mode ? (log(fmax(p, 1e-300)) - log(f)) : r;
  }
  e = group_max(e, S, tid, sync);
  badv = group_max(badv, S, tid, sync);
  // weights f0_j / max f0: the scale on which ||phi - f0||_inf is judged
  double fmx = 0.0;
  if (m.weighted) {
    for (int j = tid; j < N; j += NT) fmx = fmax(fmx, f0[j + 1]);
    fmx = group_max(fmx, S, tid, sync);
  }
  const double winv = (m.weighted && fmx > 0.0) ? 1.0 / fmx : 0.0;
  const int it = m.iters[inst];
  if (badv != 0.0) {
    if (tid == 0) { m.status[inst] |= ST_NONFINITE; m.active[inst] = 0; m.err[inst] = e; }
    return true;
  }
  const double tol_here = (act == 1) ? m.tol32 : m.tol;
  if (e <= tol_here) {
    if (tid == 0) {
      m.err[inst] = e;
      if (act == 1 && m.verify64) m.active[inst] = 2;
      else {
        m.status[inst] |= ST_CONVERGED;
        m.active[inst] = 0;
        if (m.win) atomicMin(m.win + ii, fork_key(m, ii, it, r));
      }
    }
    return true;
  }
  if (it >= m.maxit) {
    if (tid == 0) { m.status[inst] |= ST_MAXIT; m.active[inst] = 0; m.err[inst] = e; }
    return true;
  }
  // time budget, and forked paths that can no longer win (the earliest they
  // could converge is the next evaluation): one thread decides, the whole
  // group follows
  if (m.deadline || m.win) {
    if (tid == 0) {
      int stop = 0;
      if (m.deadline && global_ns() > __ldcg(m.deadline)) stop = 1;
      else if (m.win && fork_key(m, ii, it + 1, r) > *(volatile const int *)(m.win + ii)) stop = 2;
      S.stop = stop;
    }
    sync();
    const int stop = S.stop;
    if (stop) {
      if (tid == 0) {
        if (stop == 1) m.status[inst] |= ST_WATCHDOG;
        m.active[inst] = 0;
        m.err[inst] = e;
      }
      return true;
    }
  }
  // FP32 stall: below finish_tol and no halving of the error for finish_stall
  // iterations -> the FP64 propagator continues from this field with a fresh
  // history (the FP32 density's rounding noise, ~1e-7, spoils the secant pairs
  // of the small steps near convergence)
  const int rit = m.ref_it[inst];
  if (act == 1 && m.finish_stall > 0 && e < m.finish_tol && rit >= 0 && it - rit >= m.finish_stall) {
    if (tid == 0) {
      m.active[inst] = 2;
      m.status[inst] |= ST_FP64;
      m.err[inst] = e;
      m.hcount[inst] = 0;
      m.best[inst] = INFINITY;
      m.ref_err[inst] = INFINITY;
      m.ref_it[inst] = -1;
    }
    return true;
  }
  // 2. history bookkeeping (restart when the error grew by more than `grow`)
  if (tid == 0) {
    int cnt = m.hcount[inst], head = m.hhead[inst];
    double best = m.best[inst];
    const bool fresh = (it == 0) || (rit < 0);
    const bool restart = !fresh && (e > m.grow * best);
    if (restart) { cnt = 0; best = e; m.status[inst] |= ST_RESTARTED; }
    else best = fresh ? e : fmin(best, e);
    if (fresh || e < 0.5 * m.ref_err[inst]) { m.ref_err[inst] = e; m.ref_it[inst] = it; }
    const int push = !fresh && !restart;
    const int h = head;
    if (push) { head = (head + 1) % D; cnt = cnt + 1 < D ? cnt + 1 : D; }
    for (int t = 0; t < cnt; t++) S.slot[t] = ((head - 1 - t) % D + D) % D;
    S.ctl[0] = cnt; S.ctl[1] = head; S.ctl[2] = push; S.ctl[3] = h;
    m.best[inst] = best;
  }
  sync();
  const int cnt = S.ctl[0], push = S.ctl[2], h = S.ctl[3];
  if (push) {
    for (int j = tid; j < N; j += NT) {
      hdg[(long long)h * N + j] = graw[j] - gprev[j];
      hdx[(long long)h * N + j] = w[j + 1] - wprev[j];
    }
  }
  sync();
  // 3. least squares on the raw mixing residual r: new Gram row <dr_h, dr_s>
  //    and right-hand side <dr_s, r>, inner products weighted by (f0_j / max f0)^2
  //    so that nodes whose ||phi - f0|| is far below any tolerance (the walls)
  //    do not steer the extrapolation
  if (cnt > 0) {
    // one history slot at a time: two partial sums live per thread
    for (int t = 0; t < cnt; t++) {
      const double *ds_t = hdg + (long long)S.slot[t] * N;
      double pb = 0.0, pg = 0.0;
      for (int j = tid; j < N; j += NT) {
        const double wj = m.weighted ? f0[j + 1] * winv : 1.0;
        const double gv = graw[j] * wj * wj;
        const double dh = push ? hdg[(long long)h * N + j] * wj * wj : 0.0;
        const double d = ds_t[j];
        pb += d * gv;
        pg += dh * d;
      }
      const double a = warp_sum(pb), b = warp_sum(pg);
      if (lane == 0) { S.red[t][wid] = a; S.red[MIX_MAXD + t][wid] = b; }
    }
    sync();
    if (tid == 0) {
      double A[MIX_MAXD * MIX_MAXD], rhs[MIX_MAXD];
      for (int t = 0; t < cnt; t++) {
        double sb = 0.0, sg = 0.0;
        for (int q = 0; q < NW; q++) { sb += S.red[t][q]; sg += S.red[MIX_MAXD + t][q]; }
        rhs[t] = sb;
        if (push) { G[h * D + S.slot[t]] = sg; G[S.slot[t] * D + h] = sg; }
      }
      double dmax = 0.0;
      for (int t = 0; t < cnt; t++)
        for (int u = 0; u < cnt; u++) {
          A[t * cnt + u] = G[S.slot[t] * D + S.slot[u]];
          if (t == u) dmax = fmax(dmax, A[t * cnt + u]);
        }
      for (int t = 0; t < cnt; t++) A[t * cnt + t] += m.reg * dmax + 1e-300;
      small_solve(A, rhs, cnt);
      for (int t = 0; t < cnt; t++) S.gam[t] = rhs[t];
    }
    sync();
  }
  // 4. mixed residual rbar = r - sum_s gam_s dr_s (into gcur)
  for (int j = tid; j < N; j += NT) {
    double rb = graw[j];
    for (int t = 0; t < cnt; t++) rb -= S.gam[t] * hdg[(long long)S.slot[t] * N + j];
    gcur[j] = rb;
  }
  sync();
  // 5. update w <- w - sum_s gam_s dx_s + beta (1 + a (-d2/dx2)) rbar
  //    (the preconditioner acts on the step only, so FP32 rounding noise it
  //    amplifies never enters the least squares; the mixed residual is
  //    extended linearly past the first and last interior nodes, i.e. no
  //    curvature term there); beta = 1 - lk.  The step is scaled so that its
  //    f0-weighted max norm is <= clip and no node moves by more than
  //    step_cap / ds; the field is kept >= -field_floor / ds.
  const double beta = 1.0 - m.lk[inst];
  const double dsi = m.ds[ii];
  const bool graded = m.spacing && m.graded_ratio > 0.0 && m.spacing[ii] > m.graded_ratio;
  const double hf = graded ? sqrt(m.hfloor * dsi) : 0.0;  // preconditioner spacing floor
  // forked paths of this update (an instance's own path forks once, at its
  // first update number >= fork_at taken at an error <= fork_err): path f + 1
  // steps by d + beta (fork_scale[f] - 1) p, p the preconditioned residual, i.e.
  // with its own mixing parameter; staged in its own wprev
  const int nf = (m.forks > 0 && r == 0 && it + 1 >= m.fork_at && e <= m.fork_err && m.fork_it[ii] == 0)
                     ? min(m.forks, 4) : 0;
  double dm = 0.0, da = 0.0, dmf[4] = {0.0, 0.0, 0.0, 0.0}, daf[4] = {0.0, 0.0, 0.0, 0.0};
  for (int j = tid; j < N; j += NT) {
    const double gc = gcur[j];
    double lap = 0.0;
    if (j > 0 && j < N - 1) {
      const double a1 = fmax(x[j + 1] - x[j], hf), a2 = fmax(x[j + 2] - x[j + 1], hf);
      lap = ((gc - gcur[j - 1]) / a1 + (gc - gcur[j + 1]) / a2) / (0.5 * (a1 + a2));
    }
    const double pr = gc + m.precond * lap;
    double d = beta * pr;
    for (int t = 0; t < cnt; t++) d -= S.gam[t] * hdx[(long long)S.slot[t] * N + j];
    wprev[j] = d;  // staged; wprev receives the old field below
    const double wj = m.weighted ? f0[j + 1] * winv : 1.0;
    dm = fmax(dm, fabs(d) * wj);
    da = fmax(da, fabs(d));
#pragma unroll
    for (int f = 0; f < 4; f++)
      if (f < nf) {
        const double df = d + beta * (m.fork_scale[f] - 1.0) * pr;
        m.wprev[io + (f + 1) * m.rep_int + j] = df;
        dmf[f] = fmax(dmf[f], fabs(df) * wj);
        daf[f] = fmax(daf[f], fabs(df));
      }
  }
  // the step is scaled so that its f0-weighted max norm is <= clip and no node
  // moves by more than step_cap / ds (graded meshes: that bound clamps each
  // node's move instead)
  auto step_scale = [&](double vm, double va) {
    double sc = (vm > m.clip) ? m.clip / vm : 1.0;
    if (!graded && m.step_cap > 0.0 && va * sc * dsi > m.step_cap) sc = m.step_cap / (va * dsi);
    return sc;
  };
  const double lim = (graded && m.step_cap > 0.0) ? m.step_cap / dsi : INFINITY;
  auto move = [&](double v) { return fmin(fmax(v, -lim), lim); };
  dm = group_max(dm, S, tid, sync);
  da = group_max(da, S, tid, sync);
  const double scale = step_scale(dm, da);
  double scf[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int f = 0; f < 4; f++)
    if (f < nf) {
      const double vm = group_max(dmf[f], S, tid, sync);
      const double va = group_max(daf[f], S, tid, sync);
      scf[f] = step_scale(vm, va);
    }
  const double wfloor = (m.field_floor > 0.0) ? -m.field_floor / dsi : -INFINITY;
  for (int j = tid; j < N; j += NT) {
    const double wo = w[j + 1];
    const double d = wprev[j];
    wprev[j] = wo;
    gprev[j] = graw[j];
    w[j + 1] = fmax(wo + move(scale * d), wfloor);
#pragma unroll
    for (int f = 0; f < 4; f++)
      if (f < nf) {
        const long long fo = io + (f + 1) * m.rep_int;
        const double df = m.wprev[fo + j];
        m.wprev[fo + j] = wo;
        m.gprev[fo + j] = graw[j];
        m.w[no + (f + 1) * m.rep_nodes + j + 1] = fmax(wo + move(scf[f] * df), wfloor);
      }
  }
  if (nf) {
    // the rest of each forked path's state: history, Gram matrix, wall values
    // and the scalars of the instance after this update
    for (int f = 0; f < nf; f++) {
      const long long fo = io + (f + 1) * m.rep_int;
      double *hx = m.hdx + fo * D, *hg = m.hdg + fo * D;
      for (int k = tid; k < D * N; k += NT) { hx[k] = hdx[k]; hg[k] = hdg[k]; }
      const int v = inst + (f + 1) * m.base;
      double *Gf = m.gram + (long long)v * D * D;
      for (int k = tid; k < D * D; k += NT) Gf[k] = G[k];
      if (tid == 0) {
        double *wf = m.w + no + (f + 1) * m.rep_nodes;
        wf[0] = w[0];
        wf[n - 1] = w[n - 1];
        m.iters[v] = it + 1;
        m.hcount[v] = cnt;
        m.hhead[v] = S.ctl[1];
        m.err[v] = e;
        m.best[v] = m.best[inst];
        m.ref_err[v] = m.ref_err[inst];
        m.ref_it[v] = m.ref_it[inst];
        m.lk[v] = 1.0 - beta * m.fork_scale[f];
        m.status[v] = m.status[inst];
        m.active[v] = act;
      }
    }
    __threadfence();  // the forked state is complete before the caller publishes it
  }
  if (tid == 0) {
    m.iters[inst] = it + 1;
    m.hcount[inst] = cnt;
    m.hhead[inst] = S.ctl[1];
    m.err[inst] = e;
    if (m.lk_schedule) {
      double l = m.lk[inst];
      if (e < 0.03 && it > 100) l *= m.lmd;
      if (l < 1e-5) l = m.lmd;
      m.lk[inst] = l;
    }
    S.forked = nf;
    if (nf) m.fork_it[ii] = it + 1;
  }
  sync();
  return false;
}

}  // namespace scft
