// Serving loop for Poisson solves: requests (a tree, a right-hand-side seed)
// arrive at any time; an admission controller lets a request in when its
// estimated device footprint fits the memory budget, and a pool of worker
// threads runs the admitted requests concurrently -- each on its own
// per-thread default stream, so the kernels of different requests overlap
// on the device.  A worker builds the DA and the conforming plan on the
// device, forms b (uniform[-1,1] from the seed, Dirichlet rows zeroed),
// solves A x = b with the device-resident solver and keeps x for the
// caller.  When a request finishes, its memory is released and waiting
// requests are admitted in arrival order.
//
// Every stage of a request is timed (submit, admit, start, done) so the
// caller gets queueing and service latency separately.  The footprint
// estimate starts from a per-dimension bytes-per-element figure and is
// raised to the largest footprint measured so far (the worker thread's DBuf
// peak), so the budget holds for the meshes actually seen.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include "../../include/dkt_gb300.h"
#include "dkt_handles.cuh"

namespace dkt {

int pcg_solve(Plan &pl, const double *b, double *x, int precision, int max_iter, double tol, bool jacobi,
              int *iters, int *refinements, double *relres, cudaStream_t user);

__global__ void k_rhs_uniform(double *__restrict__ b, int64_t n, uint64_t seed)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t z = seed * 0xD1B54A32D192ED03ull + (uint64_t) i;
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  b[i] = 2.0 * ((double) (z >> 11) * 0x1.0p-53) - 1.0;
}
__global__ void k_zero_rows(double *__restrict__ v, const uint32_t *__restrict__ ids, int64_t nb)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) v[ids[i]] = 0.0;
}

struct SrvReq {
  int64_t id = 0;
  int dim = 0, md = 0;
  int64_t n_elem = 0;
  std::vector<uint32_t> coords;
  std::vector<uint8_t> levels;
  uint64_t seed = 0;
  double est = 0.0;
  // results
  int state = 0;   // 0 queued, 1 admitted, 2 running, 3 done
  int rc = 0;
  std::string err;
  int64_t n_nodes = 0, bytes = 0;
  int iters = 0, refinements = 0;
  double relres = 0.0;
  double t_submit = 0, t_admit = 0, t_start = 0, t_done = 0;
  std::vector<double> x;
};

struct Server {
  int workers = 1, precision = 1, max_iter = 100000, device = 0;
  double budget = 0.0, tol = 1e-10, used = 0.0;
  double bpe[5] = {0, 0, 600.0, 1200.0, 2600.0};   // bytes per element, per dim
  bool stop = false;
  int64_t next_id = 1;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<SrvReq *> queued, admitted;
  std::unordered_map<int64_t, SrvReq *> all;
  std::vector<std::thread> pool;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

  double now() const
  {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  // with m held: admit queued requests in arrival order while they fit
  void admit_locked()
  {
    while (!queued.empty()) {
      SrvReq *r = queued.front();
      const bool idle = used == 0.0;   // a request larger than the budget still runs alone
      if (!idle && used + r->est > budget) break;
      queued.pop_front();
      used += r->est;
      r->state = 1;
      r->t_admit = now();
      admitted.push_back(r);
      cv_work.notify_one();
    }
  }

  void run(SrvReq &r)
  {
    DKT_CUDA(cudaSetDevice(device));
    MemCounter &mc = mem_counter();
    const int64_t base = mc.cur;
    mc.peak = mc.cur;
    dkt_da da = nullptr;
    dkt_plan plan = nullptr;
    auto check = [&](int rc) {
      if (rc != DKT_OK) throw std::runtime_error(std::string("request failed: ") + dkt_last_error());
    };
    try {
      check(dkt_da_create(r.dim, 1, DKT_CURVE_MORTON, r.md, r.coords.data(), r.levels.data(), r.n_elem, 0, &da));
      check(dkt_plan_create_ex(da, DKT_OP_LAPLACE, nullptr, DKT_TRAVERSAL_CONFORMING, &plan));
      if (precision == 2) check(dkt_plan_set_arithmetic(plan, DKT_ARITH_FP64));
      Plan &pl = plan->pl;
      const int64_t n = pl.n_nodes;
      r.n_nodes = n;
      DBuf<double> b(n), x(n);
      k_rhs_uniform<<<grid_for(n), 256>>>(b.p, n, r.seed);
      if (pl.n_bdry > 0) k_zero_rows<<<grid_for(pl.n_bdry), 256>>>(b.p, pl.bdry.p, pl.n_bdry);
      DKT_CUDA(cudaMemsetAsync(x.p, 0, n * sizeof(double)));
      check_launch("serve_rhs");
      r.rc = pcg_solve(pl, b.p, x.p, precision == 1 ? 1 : 0, max_iter, tol, true, &r.iters, &r.refinements,
                       &r.relres, 0);
      r.x.resize(n);
      DKT_CUDA(cudaMemcpy(r.x.data(), x.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    } catch (const std::exception &e) {
      r.rc = DKT_E_INTERNAL;
      r.err = e.what();
    }
    if (plan) dkt_plan_destroy(plan);
    if (da) dkt_da_destroy(da);
    r.bytes = mc.peak - base;
  }

  void worker()
  {
    for (;;) {
      SrvReq *r = nullptr;
      {
        std::unique_lock<std::mutex> lk(m);
        cv_work.wait(lk, [&] { return stop || !admitted.empty(); });
        if (admitted.empty()) return;   // stop requested and nothing left
        r = admitted.front();
        admitted.pop_front();
        r->state = 2;
        r->t_start = now();
      }
      run(*r);
      {
        std::lock_guard<std::mutex> lk(m);
        r->t_done = now();
        r->state = 3;
        used -= r->est;
        if (used < 1e-6) used = 0.0;
        if (r->rc != DKT_E_INTERNAL && r->n_elem > 0)
          bpe[r->dim] = std::max(bpe[r->dim], 1.1 * (double) r->bytes / (double) r->n_elem);
        admit_locked();
      }
      cv_done.notify_all();
    }
  }
};

}  // namespace dkt

struct dkt_server_s {
  dkt::Server s;
};

extern "C" {

int dkt_server_create(int workers, double budget_bytes, int precision, double tol, dkt_server *out)
{
  if (!out || workers < 1 || workers > 64 || !(budget_bytes > 0) || precision < 0 || precision > 2 || !(tol > 0)) {
    return DKT_E_ARG;
  }
  dkt_server_s *h = new dkt_server_s();
  h->s.workers = workers;
  h->s.budget = budget_bytes;
  h->s.precision = precision;
  h->s.tol = tol;
  cudaGetDevice(&h->s.device);
  for (int k = 0; k < workers; k++) h->s.pool.emplace_back([h] { h->s.worker(); });
  *out = h;
  return DKT_OK;
}

int dkt_server_submit(dkt_server srv, int dim, int max_depth, const uint32_t *tree_coords, const uint8_t *tree_levels,
                      int64_t n_elem, uint64_t rhs_seed, int64_t *ticket)
{
  if (!srv || !tree_coords || !tree_levels || n_elem <= 0 || dim < 2 || dim > 4 || !ticket) return DKT_E_ARG;
  dkt::SrvReq *r = new dkt::SrvReq();
  r->dim = dim;
  r->md = max_depth;
  r->n_elem = n_elem;
  r->coords.assign(tree_coords, tree_coords + n_elem * dim);
  r->levels.assign(tree_levels, tree_levels + n_elem);
  r->seed = rhs_seed;
  dkt::Server &s = srv->s;
  {
    std::lock_guard<std::mutex> lk(s.m);
    r->id = s.next_id++;
    r->est = s.bpe[dim] * (double) n_elem;
    r->t_submit = s.now();
    s.all[r->id] = r;
    s.queued.push_back(r);
    s.admit_locked();
  }
  *ticket = r->id;
  return DKT_OK;
}

int dkt_server_wait(dkt_server srv, int64_t ticket, dkt_solve_report *rep)
{
  if (!srv) return DKT_E_ARG;
  dkt::Server &s = srv->s;
  std::unique_lock<std::mutex> lk(s.m);
  auto it = s.all.find(ticket);
  if (it == s.all.end()) return DKT_E_ARG;
  dkt::SrvReq *r = it->second;
  s.cv_done.wait(lk, [&] { return r->state == 3; });
  if (rep) {
    rep->rc = r->rc;
    rep->dim = r->dim;
    rep->n_elem = r->n_elem;
    rep->n_nodes = r->n_nodes;
    rep->iterations = r->iters;
    rep->refinements = r->refinements;
    rep->relres = r->relres;
    rep->t_submit = r->t_submit;
    rep->t_admit = r->t_admit;
    rep->t_start = r->t_start;
    rep->t_done = r->t_done;
    rep->device_bytes = r->bytes;
    rep->est_bytes = r->est;
  }
  return DKT_OK;
}

int dkt_server_solution(dkt_server srv, int64_t ticket, double *x, int64_t cap)
{
  if (!srv || !x) return DKT_E_ARG;
  dkt::Server &s = srv->s;
  std::lock_guard<std::mutex> lk(s.m);
  auto it = s.all.find(ticket);
  if (it == s.all.end() || it->second->state != 3) return DKT_E_ARG;
  const dkt::SrvReq *r = it->second;
  if (cap < (int64_t) r->x.size()) return DKT_E_ARG;
  std::copy(r->x.begin(), r->x.end(), x);
  return DKT_OK;
}

int dkt_server_error(dkt_server srv, int64_t ticket, char *buf, int capacity)
{
  if (!srv || !buf || capacity <= 0) return DKT_E_ARG;
  dkt::Server &s = srv->s;
  std::lock_guard<std::mutex> lk(s.m);
  auto it = s.all.find(ticket);
  if (it == s.all.end()) return DKT_E_ARG;
  const std::string &e = it->second->err;
  const size_t n = std::min<size_t>(e.size(), (size_t) capacity - 1);
  std::copy(e.begin(), e.begin() + n, buf);
  buf[n] = '\0';
  return DKT_OK;
}

int dkt_server_release(dkt_server srv, int64_t ticket)
{
  if (!srv) return DKT_E_ARG;
  dkt::Server &s = srv->s;
  std::lock_guard<std::mutex> lk(s.m);
  auto it = s.all.find(ticket);
  if (it == s.all.end() || it->second->state != 3) return DKT_E_ARG;
  delete it->second;
  s.all.erase(it);
  return DKT_OK;
}

void dkt_server_destroy(dkt_server srv)
{
  if (!srv) return;
  dkt::Server &s = srv->s;
  {
    std::lock_guard<std::mutex> lk(s.m);
    s.stop = true;
    // requests never admitted are dropped
    for (dkt::SrvReq *r : s.queued) { s.all.erase(r->id); delete r; }
    s.queued.clear();
  }
  s.cv_work.notify_all();
  for (std::thread &t : s.pool) t.join();
  for (auto &kv : s.all) delete kv.second;
  delete srv;
}

}  // extern "C"
