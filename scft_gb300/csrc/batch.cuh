// batch.cuh -- internal layout of a batch (shared by the runtime and the
// warm-start network; not part of the C ABI).
#pragma once
#include <chrono>
#include <vector>

#include "common.cuh"
#include "mixing.cuh"
#include "scft.h"

struct ClassPlan {
  int prec = 0, C = 1, NW = 1;
  std::vector<int> items;
  int *d_items = nullptr;
  void *scratch = nullptr;
  long long slot_elems = 0;
  int workers = 0, grid = 0, gpc = 1, head = 0;
};

struct scft_batch {
  int count = 0;
  std::vector<int> n, nsteps, rule;
  std::vector<double> ds;
  std::vector<double> spacing_ratio;  // largest / smallest element of each mesh
  std::vector<double> width;          // film width x[n-1] - x[0] of each instance
  // solves activate only the instances with d_select[i] != 0 while use_select
  int *d_select = nullptr;
  bool use_select = false;
  std::vector<long long> node_off, int_off;
  long long total_nodes = 0, total_int = 0;
  // device instance data
  int *d_n = nullptr, *d_nsteps = nullptr, *d_active = nullptr, *d_status = nullptr;
  double *d_ds = nullptr, *d_x = nullptr, *d_f0 = nullptr, *d_w = nullptr, *d_phi = nullptr;
  double *d_Q = nullptr, *d_qw = nullptr, *d_w0 = nullptr, *d_spacing = nullptr;
  long long *d_node_off = nullptr, *d_int_off = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  float last_ms = 0.f;
  int *d_heads = nullptr;
  int nheads = 0;
  std::vector<ClassPlan> plans[2];
  bool planned[2] = {false, false};
  double plan_frac[2] = {0, 0};
  int plan_paths[2] = {0, 0};
  std::vector<int> shapeC[2], shapeNW[2];
  // Anderson state
  int depth = 0;
  double *d_graw = nullptr, *d_gcur = nullptr, *d_gprev = nullptr, *d_wprev = nullptr;
  double *d_hdx = nullptr, *d_hdg = nullptr, *d_gram = nullptr, *d_err = nullptr, *d_best = nullptr;
  double *d_lk = nullptr, *d_ref_err = nullptr;
  // scratch of the scheme-general propagator (scft_batch_evaluate_scheme)
  double *d_seq = nullptr;
  long long *d_seq_off = nullptr;
  int *d_ref_it = nullptr;
  unsigned long long *d_deadline = nullptr;
  int *d_iters = nullptr, *d_hcount = nullptr, *d_hhead = nullptr, *d_nactive = nullptr;
  int *h_nactive = nullptr;
  std::vector<int> trace_active;   // unfinished instances after each graph launch of the last solve
  std::vector<double> trace_ms;    // host time since the solve started at that point
  cudaStream_t st = nullptr;
  std::vector<cudaStream_t> side;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_join;
  // Live statistics of the propagator launches inside the solve graphs: one
  // event pair and one work counter per (iteration of the graph, precision,
  // class); read after every replay, accumulated per class over one solve.
  std::vector<cudaEvent_t> ev_live;
  unsigned long long *d_work = nullptr, *h_work = nullptr;
  int live_cap = 0, live_maxc = 0;
  std::vector<double> live_ms[2], live_units[2];
  std::vector<long long> live_launches[2];
  // forked paths: per-path arrays (w, phi, Q, status, active and the Anderson
  // state) hold 1 + paths copies; d_win per instance; d_fork the per-class fork
  // queues (4 control ints + one entry per instance), initialised from h_fork
  int paths = 0;
  int *d_win = nullptr, *d_fork_it = nullptr, *d_fork = nullptr, *h_fork = nullptr;
  size_t fork_cap = 0;
  // a fused solve enqueued by scft_batch_solve_async, completed by scft_batch_wait
  bool pending = false;
  scft_solve_opts pending_opts{};
  scft::MixDev pending_mix{};
  std::chrono::steady_clock::time_point pending_start{};
};


// Device view of a batch for the propagator kernels.
scft::BatchDev batch_dev(const scft_batch *B);
