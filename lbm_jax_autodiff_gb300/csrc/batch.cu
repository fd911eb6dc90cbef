// C ABI of the batched solver (include/lbm_gb300.h, "batched instances").
//
// A batch owns one solver handle per instance (each with its own grid,
// geometry, boundary modes and population buffers) and advances all of them
// with one kernel launch per step: the launch's blocks are mapped to
// (instance, block of that instance) through a table, and every block reads
// its instance's kernel arguments from device memory.  A whole gradient
// evaluation -- forward with checkpoints, recompute, adjoint, reductions and
// optionally one Adam step on each radius -- is a fixed sequence of such
// launches, which can be captured once as a CUDA graph and replayed; the
// host rebuilds geometry between replays by rewriting the argument tables.
//
// jax_lbm has no batched driver: its examples loop over configurations in
// Python (examples/11:197-225 runs the four modes one after another).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "batch.cuh"
#include "sim_handle.cuh"

namespace lbm {

template <class St>
cudaError_t launch_step_batch(const StepArgs<float>* args, const BatchInst* inst, const int2* map,
                              int nblocks, int block, bool mrt, int src_slot, int dst_slot,
                              int extra_flags, cudaStream_t stream);
cudaError_t launch_force_finalize_batch(const BatchInst* inst, int count, int with_dj,
                                        double* samples, cudaStream_t stream);
template <class St>
cudaError_t launch_adjoint_batch(const AdjArgs<float>* args, const BatchInst* inst,
                                 const int2* map, int nblocks, int block, bool mrt,
                                 int sprev_slot, int sk_slot, int nu_in_slot, int nu_out_slot,
                                 int first, int last, cudaStream_t st);
cudaError_t launch_adjoint_pair_batch(const AdjArgs<float>* args, const BatchInst* inst,
                                      const int2* map, int nblocks, bool mrt, bool soft,
                                      int sprev_slot, int sk_slot, int nu_in_slot,
                                      int nu_out_slot, int first, int last, cudaStream_t st);
cudaError_t launch_adjoint_seed_batch(const StepArgs<float>* args, const BatchInst* inst,
                                      const int2* map, int nblocks, int block, int nu_slot,
                                      cudaStream_t st);
cudaError_t launch_zero_grad_batch(const BatchInst* inst, int count, cudaStream_t st);
cudaError_t launch_reduce_gr_batch(const BatchInst* inst, int count, cudaStream_t st);
cudaError_t launch_adam_batch(const BatchInst* inst, int count, const AdamP& p, double* opt,
                              cudaStream_t st);

namespace {

constexpr int kMinBlock = 128;   // partial buffers are sized for the smallest block
constexpr int kPairBlock = 128;  // threads (pairs) per block of k_adjoint_pair_batch

// dJ/dr partial slots of an instance of n cells: 8 per block of the smallest
// block size covers both k_adjoint_batch (8 per block) and
// k_adjoint_pair_batch (8 per 256-cell interior block, then one per list
// warp, at most n / 32 of them), plus slack for the rounding of both.
size_t gr_slots(size_t n) { return (n + kMinBlock - 1) / kMinBlock * 8 + 64; }

// f_i = value[i] on every cell
__global__ void k_fill_dirs(float* __restrict__ f, int n, Consts<float> v) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const size_t N = size_t(n);
#pragma unroll
  for (int i = 0; i < Q; ++i) f[i * N + idx] = v.w[i];
}

}  // namespace
}  // namespace lbm

struct lbm_batch {
  int count = 0;
  std::vector<lbm_sim*> sims;
  std::vector<lbm_sphere> spheres;
  bool mrt = true;
  int block = 256;
  // device tables
  int nmap = 0;
  int2* d_map = nullptr;
  // block maps of k_adjoint_pair_batch: [0] instances without, [1] with a
  // porosity blend; pmap_cap entries each (the launch grid), padded with -1
  bool pair_adjoint = false;
  int2* d_pmap[2] = {nullptr, nullptr};
  int pmap_cap[2] = {0, 0};
  int pmap_used[2] = {0, 0};
  BatchInst* d_inst = nullptr;
  StepArgs<float>* d_sargs = nullptr;
  AdjArgs<float>* d_aargs = nullptr;
  double* d_out = nullptr;   // [count][8]
  double* d_dyn = nullptr;   // [count]
  double* d_opt = nullptr;   // [count][4]: r, m, v, t
  std::vector<double*> force_part, gr_part;
  // forward-run phase (lbm_batched_run)
  int state_is_S = 0;
  int cur = 0;
  long long steps = 0;
  // gradient plan
  int plan_K = 0, plan_recompute = 0;
  unsigned long long plan_bytes = 0;
  size_t workspace_limit = 0;   // cap on the automatic plan's workspace, all instances (0: none)
  // captured gradient evaluation
  cudaStream_t gs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_N = -1, g_K = -1, g_block = -1, g_adam = -1;
  AdamP g_p{};
  double graph_seconds = 0.0;
  long long graph_launches = 0;   // kernel nodes of the captured graph
};

namespace {

long long total_cells(const lbm_batch* b) {
  long long c = 0;
  for (auto* s : b->sims) c += (long long)s->n;
  return c;
}

int build_map(lbm_batch* b) {
  std::vector<int> order(b->count);
  for (int i = 0; i < b->count; ++i) order[i] = i;
  // largest instances first: their blocks start early, small ones fill the tail
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->sims[x]->n > b->sims[y]->n; });
  std::vector<int2> map;
  for (int i : order) {
    const int nb = int((b->sims[i]->n + b->block - 1) / b->block);
    for (int j = 0; j < nb; j += kBatchChunk) map.push_back(make_int2(i, j));
  }
  cudaFree(b->d_map);
  b->d_map = nullptr;
  LBM_TRY(dev_alloc((void**)&b->d_map, map.size() * sizeof(int2)));
  LBM_TRY(cuda_check(cudaMemcpy(b->d_map, map.data(), map.size() * sizeof(int2),
                                cudaMemcpyHostToDevice),
                     "map H2D"));
  b->nmap = int(map.size());
  return LBM_OK;
}

void drop_graph(lbm_batch* b);

// Block maps of the pair adjoint from the instances' current adjoint lists:
// per instance its list blocks then its interior blocks, kPairBatchChunk per map
// entry, largest instances first.  A map only grows (padded with -1 entries)
// so the grid of a captured graph stays valid; growth drops the graph.
int build_pmaps(lbm_batch* b) {
  b->pair_adjoint = true;
  for (auto* s : b->sims)
    if ((s->g.nz % 2) != 0 || !s->spec_pairs) b->pair_adjoint = false;
  if (!b->pair_adjoint) return LBM_OK;
  std::vector<int> order(b->count);
  for (int i = 0; i < b->count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->sims[x]->n > b->sims[y]->n; });
  std::vector<int2> map[2];
  for (int i : order) {
    const lbm_sim* s = b->sims[i];
    const int soft = (s->porosity_mode == LBM_POROSITY_SOFT) ? 1 : 0;
    const int nlist = (2 * s->nspec + kPairBlock - 1) / kPairBlock;
    const int nint = int((s->n / 2 + kPairBlock - 1) / kPairBlock);
    for (int j = 0; j < nlist + nint; j += kPairBatchChunk) map[soft].push_back(make_int2(i, j));
  }
  for (int m = 0; m < 2; ++m) {
    const int need = int(map[m].size());
    if (need > b->pmap_cap[m]) {
      drop_graph(b);
      cudaFree(b->d_pmap[m]);
      b->d_pmap[m] = nullptr;
      b->pmap_cap[m] = 0;
      const int cap = need + need / 8 + 64;
      LBM_TRY(dev_alloc((void**)&b->d_pmap[m], size_t(cap) * sizeof(int2)));
      b->pmap_cap[m] = cap;
    }
    b->pmap_used[m] = need;
    if (b->pmap_cap[m] == 0) continue;
    map[m].resize(b->pmap_cap[m], make_int2(-1, 0));
    LBM_TRY(cuda_check(cudaMemcpy(b->d_pmap[m], map[m].data(), map[m].size() * sizeof(int2),
                                  cudaMemcpyHostToDevice),
                       "pair map H2D"));
  }
  return LBM_OK;
}

// Rewrite the per-instance argument tables from the handles (after geometry,
// workspace or block-size changes).  Synchronous: the tables are read by
// kernels (also by replays of a captured graph) only after this returns.
int refresh_tables(lbm_batch* b) {
  std::vector<StepArgs<float>> sa(b->count);
  std::vector<AdjArgs<float>> aa(b->count);
  std::vector<BatchInst> bi(b->count);
  std::vector<double> dyn(b->count);
  for (int i = 0; i < b->count; ++i) {
    lbm_sim* s = b->sims[i];
    fill_args<float>(s, sa[i]);
    sa[i].force_partials = b->force_part[i];
    memset(&aa[i], 0, sizeof(AdjArgs<float>));
    aa[i].s = sa[i];
    aa[i].s.flags &= ~(SF_GUARD_PRE | SF_GUARD_POST);
    BatchInst& t = bi[i];
    memset(&t, 0, sizeof(t));
    t.f0 = s->fbuf;
    t.S[0] = s->S[0];
    t.S[1] = s->S[1];
    t.nu[0] = s->nu[0];
    t.nu[1] = s->nu[1];
    t.states = static_cast<char*>(s->states);
    t.state_bytes = s->n * Q * s->st_bytes;
    t.force_part = b->force_part[i];
    t.gr_part = b->gr_part[i];
    t.ngr = int(gr_slots(s->n));
    t.gq = s->gq;
    t.ngq = s->gq ? s->nrec * Q : 0;
    t.nblk = int((s->n + b->block - 1) / b->block);
    t.out = b->d_out + 8 * i;
    t.dyn_area = b->d_dyn + i;
    dyn[i] = dyn_area(s);
  }
  LBM_TRY(cuda_check(cudaMemcpy(b->d_sargs, sa.data(), sa.size() * sizeof(sa[0]),
                                cudaMemcpyHostToDevice), "args H2D"));
  LBM_TRY(cuda_check(cudaMemcpy(b->d_aargs, aa.data(), aa.size() * sizeof(aa[0]),
                                cudaMemcpyHostToDevice), "args H2D"));
  LBM_TRY(cuda_check(cudaMemcpy(b->d_inst, bi.data(), bi.size() * sizeof(bi[0]),
                                cudaMemcpyHostToDevice), "inst H2D"));
  LBM_TRY(cuda_check(cudaMemcpy(b->d_dyn, dyn.data(), dyn.size() * sizeof(double),
                                cudaMemcpyHostToDevice), "area H2D"));
  return build_pmaps(b);
}

int require_geometry(const lbm_batch* b, const char* who) {
  for (auto* s : b->sims)
    if (!s->have_geometry) {
      std::string m = std::string(who) + ": set the instances' spheres first";
      return set_error(LBM_ERR_STATE, m.c_str());
    }
  return LBM_OK;
}

// Adjoint buffers and per-link gradient storage of every instance.
int ensure_grad_buffers(lbm_batch* b) {
  for (auto* s : b->sims) {
    for (int k = 0; k < 2; ++k)
      if (!s->nu[k]) LBM_TRY(dev_alloc(&s->nu[k], s->n * Q * s->re_bytes));
    if (!s->scal) LBM_TRY(dev_alloc((void**)&s->scal, 8 * sizeof(double)));
    if (s->gq_cap < s->nrec || !s->gq) {
      cudaFree(s->gq);
      s->gq = nullptr;
      s->gq_cap = 0;
      const int cap = s->nrec > 0 ? s->nrec : 1;
      LBM_TRY(dev_alloc((void**)&s->gq, size_t(cap) * Q * sizeof(double)));
      s->gq_cap = cap;
    }
  }
  return LBM_OK;
}

// Segment length K: as the single-instance lbm_cd_and_grad, with the
// population states of all instances counted together.
int plan_workspace(lbm_batch* b, int N, int K) {
  size_t per_state = 0, have = 0;
  for (auto* s : b->sims) {
    per_state += s->n * Q * s->st_bytes;
    have += s->states_cap * s->n * Q * s->st_bytes;
  }
  if (K <= 0) {
    size_t free_b = 0, total_b = 0;
    LBM_TRY(cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"));
    free_b += have;
    const size_t reserve = (size_t(2) << 30) + total_b / 50;
    size_t avail = free_b > reserve ? free_b - reserve : 0;
    if (b->workspace_limit && b->workspace_limit < avail) avail = b->workspace_limit;
    LBM_TRY(plan_segment(N, (long long)(avail / per_state), per_state, &K));
  }
  if (K > N) K = N;
  const int nseg = (N + K - 1) / K;
  const size_t need = size_t(nseg - 1) + size_t(K);
  for (auto* s : b->sims) {
    if (s->states_cap < need) {
      cudaFree(s->states);
      s->states = nullptr;
      s->states_cap = 0;
      LBM_TRY(dev_alloc(&s->states, need * s->n * Q * s->st_bytes));
      s->states_cap = need;
    }
    s->plan_K = K;
    s->plan_recompute = N - K;
    s->plan_bytes = need * s->n * Q * s->st_bytes;
  }
  b->plan_K = K;
  b->plan_recompute = N - K;
  b->plan_bytes = need * per_state;
  return LBM_OK;
}

int step_b(lbm_batch* b, int src, int dst, int extra, cudaStream_t st) {
  return cuda_check(launch_step_batch<float>(b->d_sargs, b->d_inst, b->d_map, b->nmap, b->block,
                                             b->mrt, src, dst, extra, st),
                    "k_step_batch launch");
}

// The launches of one gradient evaluation over n_steps with segment length K
// (and an Adam step when `adam`): the batched form of lbm_cd_and_grad.
int enqueue_grad(lbm_batch* b, int N, int K, const AdamP* adam, cudaStream_t st) {
  const int nseg = (N + K - 1) / K;
  auto ckpt = [&](int c) { return c; };
  auto stash = [&](int j) { return nseg - 2 + j; };   // j = 1..K
  auto seg_a = [&](int c) -> int {
    if (c <= 0) return 0;
    if (c >= nseg) return N;
    return N - (nseg - c) * K;
  };
  const int a_last = seg_a(nseg - 1);
  int prev = SLOT_F0, next_ck = 1;
  for (int k = 0; k < N; ++k) {
    int dst;
    if (k >= a_last) {
      dst = stash(k - a_last + 1);
    } else if (next_ck < nseg && k == seg_a(next_ck) - 1) {
      dst = ckpt(next_ck - 1);
      ++next_ck;
    } else {
      dst = (k & 1) ? SLOT_S1 : SLOT_S0;
      if (dst == prev) dst = (dst == SLOT_S0) ? SLOT_S1 : SLOT_S0;
    }
    LBM_TRY(step_b(b, prev, dst, k == 0 ? SF_COLLIDE_ONLY : 0, st));
    prev = dst;
  }
  LBM_TRY(step_b(b, prev, SLOT_NU1, SF_STREAM_ONLY | SF_FORCE, st));
  LBM_TRY(cuda_check(launch_force_finalize_batch(b->d_inst, b->count, 1, nullptr, st), "force"));
  LBM_TRY(cuda_check(launch_zero_grad_batch(b->d_inst, b->count, st), "zero"));
  LBM_TRY(cuda_check(launch_adjoint_seed_batch(b->d_sargs, b->d_inst, b->d_map, b->nmap, b->block,
                                               SLOT_NU0, st),
                     "seed"));
  int cur = 0;
  for (int c = nseg - 1; c >= 0; --c) {
    const int a0 = seg_a(c), b0 = seg_a(c + 1);
    const int slot0 = a0 == 0 ? SLOT_F0 : ckpt(c - 1);
    if (c != nseg - 1) {
      int pv = slot0;
      for (int k = a0; k < b0; ++k) {
        const int dst = stash(k - a0 + 1);
        LBM_TRY(step_b(b, pv, dst, k == 0 ? SF_COLLIDE_ONLY : 0, st));
        pv = dst;
      }
    }
    for (int k = b0 - 1; k >= a0; --k) {
      const int sprev = (k == a0) ? slot0 : stash(k - a0);
      const int nin = cur ? SLOT_NU1 : SLOT_NU0, nout = cur ? SLOT_NU0 : SLOT_NU1;
      if (b->pair_adjoint) {
        // instances without and with a porosity blend, one launch each
        for (int m = 0; m < 2; ++m)
          if (b->pmap_used[m] > 0)
            LBM_TRY(cuda_check(
                launch_adjoint_pair_batch(b->d_aargs, b->d_inst, b->d_pmap[m], b->pmap_cap[m],
                                          b->mrt, m == 1, sprev, stash(k - a0 + 1), nin, nout,
                                          k == 0, k == N - 1, st),
                "k_adjoint_pair_batch launch"));
      } else {
        LBM_TRY(cuda_check(launch_adjoint_batch<float>(b->d_aargs, b->d_inst, b->d_map, b->nmap,
                                                       b->block, b->mrt, sprev,
                                                       stash(k - a0 + 1), nin, nout, k == 0,
                                                       k == N - 1, st),
                           "k_adjoint_batch launch"));
      }
      cur = 1 - cur;
    }
  }
  LBM_TRY(cuda_check(launch_reduce_gr_batch(b->d_inst, b->count, st), "reduce"));
  if (adam) LBM_TRY(cuda_check(launch_adam_batch(b->d_inst, b->count, *adam, b->d_opt, st), "adam"));
  return LBM_OK;
}

void drop_graph(lbm_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_N = b->g_K = b->g_block = b->g_adam = -1;
}

bool same_adam(const AdamP& a, const AdamP& c) { return memcmp(&a, &c, sizeof(AdamP)) == 0; }

// Run one gradient evaluation (and Adam step) on `stream`, through the
// captured graph when use_graph.
int run_grad(lbm_batch* b, int N, int K, const AdamP* adam, int use_graph, cudaStream_t stream) {
  if (!use_graph) return enqueue_grad(b, N, K, adam, stream);
  const int want_adam = adam ? 1 : 0;
  if (!b->gexec || b->g_N != N || b->g_K != K || b->g_block != b->block ||
      b->g_adam != want_adam || (adam && !same_adam(*adam, b->g_p))) {
    drop_graph(b);
    const auto t0 = std::chrono::steady_clock::now();
    LBM_TRY(cuda_check(cudaStreamBeginCapture(b->gs, cudaStreamCaptureModeThreadLocal),
                       "begin capture"));
    const int rc = enqueue_grad(b, N, K, adam, b->gs);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->gs, &graph);
    if (rc != LBM_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    LBM_TRY(cuda_check(ec, "end capture"));
    size_t nodes = 0;
    const cudaError_t en = cudaGraphGetNodes(graph, nullptr, &nodes);
    if (en != cudaSuccess) {
      cudaGraphDestroy(graph);
      return cuda_check(en, "graph nodes");
    }
    b->graph_launches = (long long)nodes;
    const cudaError_t ei = cudaGraphInstantiate(&b->gexec, graph, 0);
    cudaGraphDestroy(graph);
    LBM_TRY(cuda_check(ei, "graph instantiate"));
    b->graph_seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    b->g_N = N;
    b->g_K = K;
    b->g_block = b->block;
    b->g_adam = want_adam;
    if (adam) b->g_p = *adam;
  }
  LBM_TRY(cuda_check(cudaEventRecord(b->ev_in, stream), "event"));
  LBM_TRY(cuda_check(cudaStreamWaitEvent(b->gs, b->ev_in, 0), "wait"));
  LBM_TRY(cuda_check(cudaGraphLaunch(b->gexec, b->gs), "graph launch"));
  LBM_TRY(cuda_check(cudaEventRecord(b->ev_out, b->gs), "event"));
  return cuda_check(cudaStreamWaitEvent(stream, b->ev_out, 0), "wait");
}

int prepare_grad(lbm_batch* b, int N, int K, const char* who) {
  if (N < 1) return set_error(LBM_ERR_ARG, "n_steps < 1");
  LBM_TRY(require_geometry(b, who));
  if (b->sims[0]->p.guard != LBM_GUARD_OFF)
    return set_error(LBM_ERR_UNSUPPORTED,
                     "batched gradient: the stability guard is not differentiated");
  LBM_TRY(ensure_grad_buffers(b));
  LBM_TRY(plan_workspace(b, N, K));
  return refresh_tables(b);
}

}  // namespace

extern "C" {

int lbm_batch_create(const lbm_params* params, int count, lbm_batch** out) {
  if (!params || !out || count < 1) return set_error(LBM_ERR_ARG, "lbm_batch_create: bad argument");
  *out = nullptr;
  for (int i = 0; i < count; ++i) {
    if (params[i].storage != LBM_F32)
      return set_error(LBM_ERR_UNSUPPORTED, "lbm_batch_create: instances use LBM_F32 storage");
    if (params[i].collision != params[0].collision || params[i].guard != params[0].guard)
      return set_error(LBM_ERR_UNSUPPORTED,
                       "lbm_batch_create: instances share the collision model and guard");
  }
  lbm_batch* b = new (std::nothrow) lbm_batch();
  if (!b) return set_error(LBM_ERR_NOMEM, "lbm_batch_create: host allocation failed");
  b->count = count;
  b->mrt = params[0].collision == LBM_MRT;
  int rc = LBM_OK;
  do {
    for (int i = 0; i < count && rc == LBM_OK; ++i) {
      lbm_sim* s = nullptr;
      rc = lbm_create(&params[i], &s);
      if (rc == LBM_OK) b->sims.push_back(s);
    }
    if (rc) break;
    b->spheres.resize(count);
    for (int i = 0; i < count && rc == LBM_OK; ++i) {
      const size_t nb = (b->sims[i]->n + kMinBlock - 1) / kMinBlock;
      double *fp = nullptr, *gp = nullptr;
      if ((rc = dev_alloc((void**)&fp, nb * 3 * sizeof(double)))) break;
      b->force_part.push_back(fp);
      if ((rc = dev_alloc((void**)&gp, gr_slots(b->sims[i]->n) * sizeof(double)))) break;
      b->gr_part.push_back(gp);
    }
    if (rc) break;
    if ((rc = dev_alloc((void**)&b->d_inst, count * sizeof(BatchInst)))) break;
    if ((rc = dev_alloc((void**)&b->d_sargs, count * sizeof(StepArgs<float>)))) break;
    if ((rc = dev_alloc((void**)&b->d_aargs, count * sizeof(AdjArgs<float>)))) break;
    if ((rc = dev_alloc((void**)&b->d_out, count * 8 * sizeof(double)))) break;
    if ((rc = cuda_check(cudaMemset(b->d_out, 0, count * 8 * sizeof(double)), "memset"))) break;
    if ((rc = dev_alloc((void**)&b->d_dyn, count * sizeof(double)))) break;
    if ((rc = dev_alloc((void**)&b->d_opt, count * 4 * sizeof(double)))) break;
    if ((rc = cuda_check(cudaStreamCreateWithFlags(&b->gs, cudaStreamNonBlocking), "stream"))) break;
    if ((rc = cuda_check(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming), "event"))) break;
    if ((rc = cuda_check(cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming), "event"))) break;
    rc = build_map(b);
  } while (0);
  if (rc) {
    lbm_batch_destroy(b);
    return rc;
  }
  *out = b;
  return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* b) {
  if (!b) return LBM_OK;
  if (b->gs) cudaStreamSynchronize(b->gs);
  drop_graph(b);
  for (auto* s : b->sims) lbm_destroy(s);
  for (auto* p : b->force_part) cudaFree(p);
  for (auto* p : b->gr_part) cudaFree(p);
  cudaFree(b->d_map);
  cudaFree(b->d_pmap[0]);
  cudaFree(b->d_pmap[1]);
  cudaFree(b->d_inst);
  cudaFree(b->d_sargs);
  cudaFree(b->d_aargs);
  cudaFree(b->d_out);
  cudaFree(b->d_dyn);
  cudaFree(b->d_opt);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->ev_out) cudaEventDestroy(b->ev_out);
  if (b->gs) cudaStreamDestroy(b->gs);
  delete b;
  return LBM_OK;
}

int lbm_batch_size(lbm_batch* b, int* count, long long* cells) {
  if (!b || !count || !cells) return set_error(LBM_ERR_ARG, "lbm_batch_size: null argument");
  *count = b->count;
  *cells = total_cells(b);
  return LBM_OK;
}

int lbm_batch_instance(lbm_batch* b, int i, lbm_sim** sim) {
  if (!b || !sim || i < 0 || i >= b->count)
    return set_error(LBM_ERR_ARG, "lbm_batch_instance: bad argument");
  *sim = b->sims[i];
  return LBM_OK;
}

int lbm_batch_set_spheres(lbm_batch* b, const lbm_sphere* spheres, void* stream) {
  if (!b || !spheres) return set_error(LBM_ERR_ARG, "lbm_batch_set_spheres: null argument");
  for (int i = 0; i < b->count; ++i) {
    LBM_TRY(lbm_set_geometry_sphere(b->sims[i], &spheres[i], stream));
    b->spheres[i] = spheres[i];
  }
  return refresh_tables(b);
}

int lbm_batch_set_equilibrium(lbm_batch* b, void* stream) {
  if (!b) return set_error(LBM_ERR_ARG, "lbm_batch_set_equilibrium: null handle");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (auto* s : b->sims) {
    // f_eq(1, (U, 0, 0)) of the reference's initial state (examples/10:152-154)
    Consts<float> v;
    Consts<double> Kd;
    fill_consts<double>(s->p, Kd);
    const double U = s->p.inlet_velocity[0];
    for (int i = 0; i < Q; ++i) {
      const double eu = ex(i) * U;
      v.w[i] = float(Kd.w[i] * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * U * U));
    }
    const int n = int(s->n);
    k_fill_dirs<<<(n + 255) / 256, 256, 0, st>>>(static_cast<float*>(s->fbuf), n, v);
    LBM_TRY(cuda_check(cudaGetLastError(), "fill"));
    s->state_is_S = 0;
    s->steps = 0;
    s->fbuf_step = 0;
  }
  b->state_is_S = 0;
  b->steps = 0;
  return LBM_OK;
}

int lbm_batch_set_state(lbm_batch* b, int i, const void* f, void* stream) {
  if (!b || i < 0 || i >= b->count) return set_error(LBM_ERR_ARG, "lbm_batch_set_state: bad index");
  LBM_TRY(lbm_set_state(b->sims[i], f, stream));
  b->state_is_S = 0;
  b->steps = 0;
  return LBM_OK;
}

int lbm_batched_run(lbm_batch* b, int n_steps, int sample_every, double* samples, void* stream) {
  if (!b) return set_error(LBM_ERR_ARG, "lbm_batched_run: null handle");
  if (n_steps < 0) return set_error(LBM_ERR_ARG, "lbm_batched_run: n_steps < 0");
  if (sample_every < 0 || (sample_every > 0 && !samples))
    return set_error(LBM_ERR_ARG, "lbm_batched_run: sample_every > 0 needs a samples buffer");
  LBM_TRY(check_align(samples, 8, "samples"));
  LBM_TRY(require_geometry(b, "lbm_batched_run"));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto want_sample = [&](long long k_global, long long k0) -> long long {
    if (sample_every <= 0) return -1;
    const long long rel = k_global - k0;
    if (rel <= 0 || rel % sample_every) return -1;
    return rel / sample_every - 1;
  };
  const long long k0 = b->steps;
  const int S[2] = {SLOT_S0, SLOT_S1};
  for (int L = 1; L <= n_steps; ++L) {
    if (!b->state_is_S) {
      LBM_TRY(step_b(b, SLOT_F0, S[b->cur], SF_COLLIDE_ONLY, st));
      b->state_is_S = 1;
    } else {
      const long long si = want_sample(b->steps, k0);
      LBM_TRY(step_b(b, S[b->cur], S[1 - b->cur], si >= 0 ? SF_FORCE : 0, st));
      if (si >= 0)
        LBM_TRY(cuda_check(launch_force_finalize_batch(b->d_inst, b->count, 0,
                                                       samples + size_t(si) * 4 * b->count, st),
                           "force"));
      b->cur = 1 - b->cur;
    }
    b->steps += 1;
  }
  const long long si = want_sample(b->steps, k0);
  if (si >= 0) {
    // sample after the last step: stream-only pass into the (no longer needed)
    // f_0 buffer, state unchanged -- as lbm_run
    LBM_TRY(step_b(b, S[b->cur], SLOT_F0, SF_STREAM_ONLY | SF_FORCE, st));
    LBM_TRY(cuda_check(launch_force_finalize_batch(b->d_inst, b->count, 0,
                                                   samples + size_t(si) * 4 * b->count, st),
                       "force"));
  }
  for (auto* s : b->sims) {
    s->state_is_S = b->state_is_S;
    s->cur = b->cur;
    s->steps = b->steps;
    if (si >= 0) s->fbuf_step = b->steps;   // the last sample pass wrote f into f_0's buffer
  }
  return LBM_OK;
}

int lbm_batch_cd_and_grad(lbm_batch* b, int n_steps, int checkpoint_every, int use_graph,
                          double* cd_host, double* dcd_dr_host, void* stream) {
  if (!b || !cd_host || !dcd_dr_host)
    return set_error(LBM_ERR_ARG, "lbm_batch_cd_and_grad: null argument");
  if (b->state_is_S)
    return set_error(LBM_ERR_STATE,
                     "lbm_batch_cd_and_grad: needs the initial state; call lbm_batch_set_equilibrium");
  LBM_TRY(prepare_grad(b, n_steps, checkpoint_every, "lbm_batch_cd_and_grad"));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LBM_TRY(run_grad(b, n_steps, b->plan_K, nullptr, use_graph, st));
  std::vector<double> h(size_t(b->count) * 8);
  LBM_TRY(cuda_check(cudaMemcpyAsync(h.data(), b->d_out, h.size() * sizeof(double),
                                     cudaMemcpyDeviceToHost, st), "D2H"));
  LBM_TRY(cuda_check(cudaStreamSynchronize(st), "sync"));
  for (int i = 0; i < b->count; ++i) {
    cd_host[i] = h[8 * i + 3];
    dcd_dr_host[i] = h[8 * i + 5];
  }
  return LBM_OK;
}

int lbm_batch_optimize(lbm_batch* b, int n_iters, int n_steps, int checkpoint_every,
                       const lbm_adam* opt, int use_graph, double* r_hist, double* loss_hist,
                       double* cd_hist, double* grad_hist, void* stream) {
  if (!b || !opt || n_iters < 0) return set_error(LBM_ERR_ARG, "lbm_batch_optimize: bad argument");
  if (!(opt->lr > 0.0) || !(opt->r_min > 0.0) || !(opt->r_max >= opt->r_min))
    return set_error(LBM_ERR_ARG, "lbm_batch_optimize: lr > 0 and 0 < r_min <= r_max required");
  if (b->state_is_S)
    return set_error(LBM_ERR_STATE,
                     "lbm_batch_optimize: needs the initial state; call lbm_batch_set_equilibrium");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  AdamP p;
  memset(&p, 0, sizeof(p));
  p.lr = opt->lr;
  p.b1 = opt->b1;
  p.b2 = opt->b2;
  p.eps = opt->eps;
  p.r_min = opt->r_min;
  p.r_max = opt->r_max;
  p.target = opt->loss == LBM_LOSS_TARGET_CD ? 1 : 0;
  p.target_cd = opt->target_cd;
  std::vector<double> o(size_t(b->count) * 4, 0.0);
  for (int i = 0; i < b->count; ++i) o[4 * i] = b->spheres[i].radius;
  LBM_TRY(cuda_check(cudaMemcpy(b->d_opt, o.data(), o.size() * sizeof(double),
                                cudaMemcpyHostToDevice), "opt H2D"));
  std::vector<double> h(size_t(b->count) * 8);
  for (int it = 0; it < n_iters; ++it) {
    LBM_TRY(prepare_grad(b, n_steps, checkpoint_every, "lbm_batch_optimize"));
    LBM_TRY(run_grad(b, n_steps, b->plan_K, &p, use_graph, st));
    LBM_TRY(cuda_check(cudaMemcpyAsync(h.data(), b->d_out, h.size() * sizeof(double),
                                       cudaMemcpyDeviceToHost, st), "D2H"));
    LBM_TRY(cuda_check(cudaMemcpyAsync(o.data(), b->d_opt, o.size() * sizeof(double),
                                       cudaMemcpyDeviceToHost, st), "D2H"));
    LBM_TRY(cuda_check(cudaStreamSynchronize(st), "sync"));
    for (int i = 0; i < b->count; ++i) {
      const size_t j = size_t(it) * b->count + i;
      if (r_hist) r_hist[j] = b->spheres[i].radius;
      if (loss_hist) loss_hist[j] = h[8 * i + 6];
      if (cd_hist) cd_hist[j] = h[8 * i + 3];
      if (grad_hist) grad_hist[j] = h[8 * i + 7];
    }
    // geometry of the updated radii for the next evaluation
    for (int i = 0; i < b->count; ++i) {
      lbm_sphere sp = b->spheres[i];
      sp.radius = o[4 * i];
      LBM_TRY(lbm_set_geometry_sphere(b->sims[i], &sp, stream));
      b->spheres[i] = sp;
    }
    LBM_TRY(refresh_tables(b));
  }
  return LBM_OK;
}

int lbm_batch_get_radii(lbm_batch* b, double* radii_host) {
  if (!b || !radii_host) return set_error(LBM_ERR_ARG, "lbm_batch_get_radii: null argument");
  for (int i = 0; i < b->count; ++i) radii_host[i] = b->spheres[i].radius;
  return LBM_OK;
}

int lbm_batch_set_block(lbm_batch* b, int block) {
  if (!b || (block != 128 && block != 256))
    return set_error(LBM_ERR_ARG, "lbm_batch_set_block: 128 or 256 threads");
  if (block == b->block) return LBM_OK;
  b->block = block;
  drop_graph(b);
  LBM_TRY(build_map(b));
  for (auto* s : b->sims)
    if (!s->have_geometry) return LBM_OK;
  return refresh_tables(b);
}

int lbm_batch_autotune(lbm_batch* b, int probe_steps, int n_steps, int* block_out,
                       int* checkpoint_out, void* stream) {
  if (!b || !block_out || !checkpoint_out || probe_steps < 2 || n_steps < 1)
    return set_error(LBM_ERR_ARG, "lbm_batch_autotune: bad argument");
  if (b->state_is_S)
    return set_error(LBM_ERR_STATE,
                     "lbm_batch_autotune: needs the initial state; call lbm_batch_set_equilibrium");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  LBM_TRY(cuda_check(cudaEventCreate(&e0), "event"));
  LBM_TRY(cuda_check(cudaEventCreate(&e1), "event"));
  const int cand[2] = {128, 256};
  float best = 1e30f;
  int best_block = b->block;
  int rc = LBM_OK;
  for (int c = 0; c < 2 && rc == LBM_OK; ++c) {
    if ((rc = lbm_batch_set_block(b, cand[c]))) break;
    // a short gradient evaluation (probe_steps forward + adjoint) per shape,
    // timed after one untimed run
    if ((rc = prepare_grad(b, probe_steps, probe_steps, "lbm_batch_autotune"))) break;
    if ((rc = run_grad(b, probe_steps, probe_steps, nullptr, 0, st))) break;
    if ((rc = cuda_check(cudaEventRecord(e0, st), "event"))) break;
    if ((rc = run_grad(b, probe_steps, probe_steps, nullptr, 0, st))) break;
    if ((rc = cuda_check(cudaEventRecord(e1, st), "event"))) break;
    if ((rc = cuda_check(cudaEventSynchronize(e1), "sync"))) break;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      best_block = cand[c];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  LBM_TRY(rc);
  LBM_TRY(lbm_batch_set_block(b, best_block));
  // checkpoint interval: the longest segment the free device memory holds
  // (every shorter one recomputes more steps for the same adjoint work)
  LBM_TRY(prepare_grad(b, n_steps, 0, "lbm_batch_autotune"));
  *block_out = b->block;
  *checkpoint_out = b->plan_K;
  return LBM_OK;
}

int lbm_batch_get_plan(lbm_batch* b, int* block, int* segment_steps, int* recomputed_steps,
                       unsigned long long* workspace_bytes, double* graph_build_seconds) {
  if (!b || !block || !segment_steps || !recomputed_steps || !workspace_bytes ||
      !graph_build_seconds)
    return set_error(LBM_ERR_ARG, "lbm_batch_get_plan: null argument");
  *block = b->block;
  *segment_steps = b->plan_K;
  *recomputed_steps = b->plan_recompute;
  *workspace_bytes = b->plan_bytes;
  *graph_build_seconds = b->graph_seconds;
  return LBM_OK;
}

int lbm_batch_set_workspace_limit(lbm_batch* b, unsigned long long max_bytes) {
  if (!b) return set_error(LBM_ERR_ARG, "lbm_batch_set_workspace_limit: null handle");
  b->workspace_limit = size_t(max_bytes);
  return LBM_OK;
}

int lbm_batch_graph_launches(lbm_batch* b, long long* launches) {
  if (!b || !launches) return set_error(LBM_ERR_ARG, "lbm_batch_graph_launches: null argument");
  *launches = b->graph_launches;
  return LBM_OK;
}

}  // extern "C"
