// Emulation of the reference's function-static parent buffer.
//
// fem::matvec interpolates a hanging leaf's missing values from a parent
// buffer that is function-static (FEM/include/matvec.h:283): it refills only
// the slots that hold a parent node of level L-1 (matvec.h:415-431), applies
// IKD_Parent2Child in place to all slots (matvec.h:450), and reads the result
// at the leaf's unfilled ranks (matvec.h:454-456).  A slot it does not refill
// keeps the value the previous hanging leaf left there, so for some meshes
// (the reference then reports "parent is missing needed nodes",
// matvec.h:443-447) a leaf reads values of earlier leaves.  The buffer state
// after hanging leaf g is S_g = IP_g * merge(fresh_g, S_{g-1}), linear in the
// input vector.  Only the slots that reach an unfilled rank with nonzero
// weight matter; this file finds that dependency closure once per plan (host,
// backward sweep over the hanging leaves in traversal order), splits it into
// independent runs of consecutive hanging leaves, and evaluates each run per
// product with one thread walking it in order.  The leaf kernels then read
// the run results in place of the unrefilled slots.
#include <algorithm>
#include <array>
#include <cmath>
#include <vector>
#include "dkt_internal.cuh"

namespace dkt {

// Host analysis.  ip: [2][M][M] child interpolation (A[k*M+j]: parent k -> child j).
void stale_setup(Plan &pl, const std::vector<double> &ip, cudaStream_t s)
{
  pl.st_ready = false;
  pl.stale_slots = 0;
  pl.st_start = 0;
  const int64_t H = pl.n_hang, NL = pl.n_leaf;
  if (H == 0 || pl.conforming) return;
  const int npe = pl.npe, M = pl.order + 1, dim = pl.dim, nc = 1 << dim;
  std::vector<uint32_t> info(NL);
  std::vector<int32_t> hidx(NL), p2n((size_t) npe * H);
  std::vector<uint32_t> fill((size_t) 3 * H);
  DKT_CUDA(cudaMemcpyAsync(info.data(), pl.info.p, NL * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaMemcpyAsync(hidx.data(), pl.hidx.p, NL * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaMemcpyAsync(p2n.data(), pl.p2n.p, (size_t) npe * H * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaMemcpyAsync(fill.data(), pl.fill.p, (size_t) 3 * H * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  DKT_CUDA(cudaStreamSynchronize(s));
  std::vector<uint8_t> child(H);
  for (int64_t i = 0; i < NL; i++)
    if (hidx[i] >= 0) child[hidx[i]] = (uint8_t) ((info[i] >> 8) & 0xFFu);
  // W[c][r][q]: weight of parent slot q on child rank r
  std::vector<double> W((size_t) nc * npe * npe);
  for (int c = 0; c < nc; c++)
    for (int r = 0; r < npe; r++)
      for (int q = 0; q < npe; q++) {
        double w = 1.0;
        int rr = r, qq = q;
        for (int d = 0; d < dim; d++) {
          const int rd = rr % M, qd = qq % M;
          rr /= M;
          qq /= M;
          w *= ip[(size_t) ((c >> d) & 1) * M * M + qd * M + rd];
        }
        W[((size_t) c * npe + r) * npe + q] = w;
      }
  auto Wv = [&](int c, int r, int q) { return W[((size_t) c * npe + r) * npe + q]; };
  auto filled = [&](int64_t h, int r) { return (fill[(size_t) h * 3 + (r >> 5)] >> (r & 31)) & 1u; };
  auto stale = [&](int64_t h, int q) { return p2n[(size_t) h * npe + q] < 0; };
  // need[g]: slots of S_g that later leaves read (bit set per slot)
  std::vector<std::array<uint32_t, 3>> need(H, {0u, 0u, 0u});
  std::vector<std::array<uint32_t, 3>> hazard(H, {0u, 0u, 0u});
  int64_t n_hazard_slots = 0;
  for (int64_t h = 0; h < H; h++) {
    for (int q = 0; q < npe; q++) {
      if (!stale(h, q)) continue;
      bool hz = false;
      for (int r = 0; r < npe && !hz; r++)
        if (!filled(h, r) && Wv(child[h], r, q) != 0.0) hz = true;
      if (hz) {
        hazard[h][q >> 5] |= 1u << (q & 31);
        n_hazard_slots++;
        if (h > 0) need[h - 1][q >> 5] |= 1u << (q & 31);
        else pl.st_start++;
      }
    }
  }
  pl.stale_slots = n_hazard_slots;
  if (n_hazard_slots == 0) return;
  // backward closure: an entry (g, q) needs (g-1, q') for stale q' with weight
  for (int64_t g = H - 1; g >= 0; g--) {
    for (int q = 0; q < npe; q++) {
      if (!((need[g][q >> 5] >> (q & 31)) & 1u)) continue;
      for (int q2 = 0; q2 < npe; q2++) {
        if (!stale(g, q2) || Wv(child[g], q, q2) == 0.0) continue;
        if (g > 0) need[g - 1][q2 >> 5] |= 1u << (q2 & 31);
        else pl.st_start++;
      }
    }
  }
  // Entries in increasing g, grouped by g; groups of consecutive g form runs
  // (independent of each other).  Terms are split into fresh ones (a node's
  // input value) and stale ones (an entry of the previous group).
  std::vector<int32_t> ent_base(H, -1);
  std::vector<int32_t> frow(1, 0), fidx, srow(1, 0), sidx;
  std::vector<double> fw, sw;
  std::vector<int32_t> gstart;     // entry offset of every group, plus the end
  std::vector<int32_t> runs;       // pairs [first group, end group)
  std::vector<int32_t> gchild;     // order 2: child number of every group
  std::vector<uint32_t> gmask;     // order 2: need[3], take[3] of every group
  int32_t n_ent = 0;
  int64_t prev_g = -2;
  for (int64_t g = 0; g < H; g++) {
    const bool any = need[g][0] | need[g][1] | need[g][2];
    if (!any) continue;
    if (g != prev_g + 1) {
      if (!runs.empty()) runs.push_back((int32_t) gstart.size());
      runs.push_back((int32_t) gstart.size());
    }
    prev_g = g;
    gstart.push_back(n_ent);
    ent_base[g] = n_ent;
    gchild.push_back(child[g]);
    {
      uint32_t take[3] = {0u, 0u, 0u};
      if (g > 0)
        for (int q2 = 0; q2 < npe; q2++)
          if (stale(g, q2) && ((need[g - 1][q2 >> 5] >> (q2 & 31)) & 1u)) take[q2 >> 5] |= 1u << (q2 & 31);
      for (int w = 0; w < 3; w++) gmask.push_back(need[g][w]);
      for (int w = 0; w < 3; w++) gmask.push_back(take[w]);
    }
    for (int q = 0; q < npe; q++) {
      if (!((need[g][q >> 5] >> (q & 31)) & 1u)) continue;
      n_ent++;
      for (int q2 = 0; q2 < npe; q2++) {
        const double w = Wv(child[g], q, q2);
        if (w == 0.0) continue;
        if (!stale(g, q2)) {
          fidx.push_back(p2n[(size_t) g * npe + q2]);
          fw.push_back(w);
        } else if (g > 0 && ent_base[g - 1] >= 0) {
          int32_t id = ent_base[g - 1];
          for (int k = 0; k < q2; k++) id += (need[g - 1][k >> 5] >> (k & 31)) & 1u;
          sidx.push_back(id);
          sw.push_back(w);
        }
        // g == 0: the slot holds the buffer's initial contents (zero)
      }
      frow.push_back((int32_t) fidx.size());
      srow.push_back((int32_t) sidx.size());
    }
  }
  if (!runs.empty()) runs.push_back((int32_t) gstart.size());
  gstart.push_back(n_ent);
  {
    // longest runs first: the chain kernels hand runs out in this order
    std::vector<std::pair<int32_t, int32_t>> rp;
    for (size_t k = 0; k + 1 < runs.size(); k += 2) rp.emplace_back(runs[k], runs[k + 1]);
    std::stable_sort(rp.begin(), rp.end(), [&](const std::pair<int32_t, int32_t> &a, const std::pair<int32_t, int32_t> &b) {
      return gstart[a.second] - gstart[a.first] > gstart[b.second] - gstart[b.first];
    });
    for (size_t k = 0; k < rp.size(); k++) { runs[2 * k] = rp[k].first; runs[2 * k + 1] = rp[k].second; }
  }
  // per hazard leaf: entry id of (h-1, q) for each slot it reads stale
  std::vector<int32_t> hz_off(H, -1), hz_tab;
  for (int64_t h = 0; h < H; h++) {
    if (!(hazard[h][0] | hazard[h][1] | hazard[h][2]) || h == 0) continue;
    hz_off[h] = (int32_t) (hz_tab.size() / npe);
    for (int q = 0; q < npe; q++) {
      int32_t id = -1;
      if (stale(h, q) && ((need[h - 1][q >> 5] >> (q & 31)) & 1u)) {
        id = ent_base[h - 1];
        for (int k = 0; k < q; k++) id += (need[h - 1][k >> 5] >> (k & 31)) & 1u;
      }
      hz_tab.push_back(id);
    }
  }
  pl.st_n_ent = n_ent;
  pl.st_n_runs = (int64_t) runs.size() / 2;
  pl.st_max_run_groups = pl.st_max_run_ents = 0;
  for (size_t k = 0; k + 1 < runs.size(); k += 2) {
    pl.st_max_run_groups = std::max<int64_t>(pl.st_max_run_groups, runs[k + 1] - runs[k]);
    pl.st_max_run_ents = std::max<int64_t>(pl.st_max_run_ents, gstart[runs[k + 1]] - gstart[runs[k]]);
  }
  // keep every upload non-empty
  if (fidx.empty()) { fidx.push_back(0); fw.push_back(0.0); }
  if (sidx.empty()) { sidx.push_back(0); sw.push_back(0.0); }
  if (runs.empty()) runs.push_back(0);
  if (hz_tab.empty()) hz_tab.push_back(-1);
  pl.st_row.upload(frow.data(), frow.size(), s);
  pl.st_idx.upload(fidx.data(), fidx.size(), s);
  pl.st_w.upload(fw.data(), fw.size(), s);
  pl.st_srow.upload(srow.data(), srow.size(), s);
  pl.st_sidx.upload(sidx.data(), sidx.size(), s);
  pl.st_sw.upload(sw.data(), sw.size(), s);
  pl.st_gstart.upload(gstart.data(), gstart.size(), s);
  // Order 2 walks each group as P_c applied axis by axis to the previous
  // group's values: valid when the child interpolation copies parent nodes 0
  // and 1 in its outer rows and the second child is the mirror image.
  pl.st_tp = false;
  if (M == 3 && !gchild.empty()) {
    const double *a = ip.data(), *b = ip.data() + 9;
    bool ok = a[0] == 1 && a[3] == 0 && a[6] == 0 && a[2] == 0 && a[5] == 1 && a[8] == 0;
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) ok = ok && b[k * 3 + j] == a[(2 - k) * 3 + (2 - j)];
    if (ok) {
      pl.st_tp = true;
      pl.st_pint[0] = a[1];
      pl.st_pint[1] = a[4];
      pl.st_pint[2] = a[7];
      pl.st_gchild.upload(gchild.data(), gchild.size(), s);
      pl.st_gmask.upload(gmask.data(), gmask.size(), s);
    }
  }
  pl.st_runs.upload(runs.data(), runs.size(), s);
  pl.st_f.alloc(std::max<int64_t>(n_ent, 1));
  pl.st_hzoff.upload(hz_off.data(), hz_off.size(), s);
  // leaves that read stale slots: the tiled kernel leaves them to a second,
  // small launch that runs after the chain (info bit 27 marks them)
  std::vector<int32_t> hl;
  for (int64_t i = 0; i < NL; i++)
    if (hidx[i] >= 0 && hz_off[hidx[i]] >= 0) {
      hl.push_back((int32_t) i);
      info[i] |= 1u << 27;
    }
  pl.st_n_hleaf = (int64_t) hl.size();
  if (hl.empty()) hl.push_back(0);
  pl.st_hleaves.upload(hl.data(), hl.size(), s);
  DKT_CUDA(cudaMemcpyAsync(pl.info.p, info.data(), NL * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  pl.st_hztab.upload(hz_tab.data(), hz_tab.size(), s);
  pl.st_v.alloc(std::max<int64_t>(n_ent, 1));
  pl.st_vq.alloc(std::max<int64_t>(n_ent, 1));
  DKT_CUDA(cudaStreamSynchronize(s));
  pl.st_ready = true;
}

// Fresh part of every entry: independent, one thread each.
template <bool FIXED>
__global__ void k_stale_fresh(int64_t n_ent, const int32_t *__restrict__ row, const int32_t *__restrict__ idx,
                              const double *__restrict__ w, const double *__restrict__ x,
                              const long long *__restrict__ xq, double *__restrict__ f)
{
  const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_ent) return;
  double acc = 0.0;
  for (int32_t k = row[e]; k < row[e + 1]; k++) {
    const int32_t j = idx[k];
    acc += w[k] * (FIXED ? (double) xq[j] : x[j]);
  }
  f[e] = acc;
}

// The chained part: one block per run.  The run is cut into chunks of
// consecutive groups (at most CH_E entries and ch_t stale terms); the block
// stages a chunk's fresh parts and terms in shared memory with coalesced
// loads, one warp walks the groups in order (lanes split a group's entries;
// every term refers to the previous group, whose values are in shared
// memory), then the block writes the chunk's values out.  The walk touches
// shared memory only, so a step costs a few shared-memory latencies.
constexpr int CH_E = 256;      // entries per chunk
constexpr int CH_G = 128;      // groups per chunk
constexpr int CH_THREADS = 128;
static_assert(CH_G == CH_THREADS, "one group test per thread");

template <bool FIXED>
__global__ void __launch_bounds__(CH_THREADS) k_stale_chain(
    const int32_t *__restrict__ runs, int64_t n_runs, const int32_t *__restrict__ gstart,
    const int32_t *__restrict__ srow, const int32_t *__restrict__ sidx, const double *__restrict__ sw,
    const double *__restrict__ f, double *__restrict__ v, long long *__restrict__ vq, int ch_t, int max_grp)
{
  extern __shared__ __align__(16) unsigned char smem[];
  double *wS = reinterpret_cast<double *>(smem);            // [ch_t]
  double *fS = wS + ch_t;                                   // [CH_E]
  double *vals = fS + CH_E;                                 // [CH_E]
  double *carry = vals + CH_E;                              // [max_grp]
  int32_t *iS = reinterpret_cast<int32_t *>(carry + max_grp);   // [ch_t]
  int32_t *rS = iS + ch_t;                                  // [CH_E + 1]
  int32_t *gS = rS + CH_E + 1;                              // [CH_G + 1]
  for (int64_t run = blockIdx.x; run < n_runs; run += gridDim.x) {
  const int32_t g_end = runs[2 * run + 1];
  int32_t g0 = runs[2 * run];
  int32_t carry_base = 0;   // entry id of carry[0]
  while (g0 < g_end) {
    const int32_t e0 = gstart[g0], t0 = srow[e0];
    // chunk length: the groups [g0, g0 + cg) that fit (monotone test)
    int ok = 0;
    for (int t = threadIdx.x; t < CH_G; t += CH_THREADS) {
      const int32_t g = g0 + t;
      if (g < g_end) {
        const int32_t ee = gstart[g + 1];
        if (ee - e0 <= CH_E && srow[ee] - t0 <= ch_t) ok++;
      }
    }
    const int cg_raw = __syncthreads_count(ok);   // CH_G == CH_THREADS: ok is 0 or 1
    const int cg = cg_raw > 0 ? cg_raw : 1;
    const int32_t e1 = gstart[g0 + cg], t1 = srow[e1];
    for (int k = threadIdx.x; k <= cg; k += CH_THREADS) gS[k] = gstart[g0 + k] - e0;
    for (int32_t e = threadIdx.x; e < e1 - e0; e += CH_THREADS) {
      fS[e] = f[e0 + e];
      rS[e] = srow[e0 + e] - t0;
    }
    if (threadIdx.x == 0) rS[e1 - e0] = t1 - t0;
    for (int32_t k = threadIdx.x; k < t1 - t0; k += CH_THREADS) {
      iS[k] = sidx[t0 + k];
      wS[k] = sw[t0 + k];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      for (int j = 0; j < cg; j++) {
        const int ge0 = gS[j], ne = gS[j + 1] - ge0;
        if (ne <= 16) {
          // two lanes per entry, each summing every other term, then one shuffle
          const int e = ge0 + (lane >> 1);
          const bool on = (lane >> 1) < ne;
          double acc = 0.0;
          if (on) {
            const int k1 = rS[e + 1];
            if (j == 0) {
              for (int k = rS[e] + (lane & 1); k < k1; k += 2) acc += wS[k] * carry[iS[k] - carry_base];
            } else {
#pragma unroll 4
              for (int k = rS[e] + (lane & 1); k < k1; k += 2) acc += wS[k] * vals[iS[k] - e0];
            }
          }
          acc += __shfl_xor_sync(0xffffffffu, acc, 1);
          if (on && !(lane & 1)) vals[e] = fS[e] + acc;
        } else {
          for (int e = ge0 + lane; e < ge0 + ne; e += 32) {
            double acc = fS[e];
            if (j == 0) {
              for (int k = rS[e]; k < rS[e + 1]; k++) acc += wS[k] * carry[iS[k] - carry_base];
            } else {
#pragma unroll 4
              for (int k = rS[e]; k < rS[e + 1]; k++) acc += wS[k] * vals[iS[k] - e0];
            }
            vals[e] = acc;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
    for (int32_t e = threadIdx.x; e < e1 - e0; e += CH_THREADS) {
      const double a = vals[e];
      v[e0 + e] = a;
      if (FIXED) vq[e0 + e] = __double2ll_rn(a);
    }
    // the last group's values become the carry of the next chunk
    const int32_t lb = gS[cg - 1];
    for (int32_t e = lb + threadIdx.x; e < gS[cg]; e += CH_THREADS) carry[e - lb] = vals[e];
    carry_base = e0 + lb;
    __syncthreads();
    g0 += cg;
  }
  }
}

// Order-2 chained part.  A group's stale terms are the child interpolation
// P_c (x) .. (x) P_c applied to the previous group's values, so instead of
// per-entry term lists the walk applies P_c axis by axis: the previous
// group's values go to the slots it takes (all other slots zero), one lane
// per line of three slots applies the 1D interpolation along each axis, and
// every needed slot's result plus the entry's fresh part is the entry's
// value.  One block per run; chunks of consecutive groups (their child
// numbers, slot masks and fresh parts) are staged in shared memory by the
// whole block and walked by warp 0.
constexpr int TP_G = 128;        // groups per chunk
constexpr int TP_E = 4096;       // entries per chunk
constexpr int TP_THREADS = 128;
static_assert(TP_G == TP_THREADS, "one group test per thread");

// parent -> child along one axis (child bit cb): the outer rows copy parent
// nodes, the middle row is (pa, pb, pc) (mirrored for the second child)
__device__ __forceinline__ void ip_line(double &a, double &b, double &c, double pa, double pb, double pc, bool cb)
{
  const double y0 = cb ? b : a, y2 = cb ? c : b;
  const double y1 = fma(pc, cb ? a : c, fma(pb, b, pa * (cb ? c : a)));
  a = y0;
  b = y1;
  c = y2;
}

template <int DIM>
__global__ void __launch_bounds__(TP_THREADS) k_stale_chain_tp(
    const int32_t *__restrict__ runs, int64_t n_runs, const int32_t *__restrict__ gstart,
    const int32_t *__restrict__ gchild, const uint32_t *__restrict__ gmask, const double *__restrict__ f,
    double *__restrict__ v, double pa, double pb, double pc)
{
  constexpr int NPE = DIM == 2 ? 9 : (DIM == 3 ? 27 : 81), NL = NPE / 3;
  __shared__ double fS[TP_E];
  __shared__ double m[NPE], prevS[NPE];
  __shared__ uint32_t mS[TP_G * 6];
  __shared__ int32_t cS[TP_G], gS[TP_G + 1];
  for (int64_t run = blockIdx.x; run < n_runs; run += gridDim.x) {
  const int32_t g_end = runs[2 * run + 1];
  int32_t g0 = runs[2 * run];
  while (g0 < g_end) {
    const int32_t e0 = gstart[g0];
    // chunk: the groups [g0, g0 + cg) whose entries fit (monotone test)
    const int32_t gt = g0 + (int32_t) threadIdx.x;
    const int ok = (gt < g_end && gstart[gt + 1] - e0 <= TP_E) ? 1 : 0;
    const int cg_raw = __syncthreads_count(ok);
    const int cg = cg_raw > 0 ? cg_raw : 1;   // a group has at most NPE < TP_E entries
    const int32_t e1 = gstart[g0 + cg];
    for (int k = threadIdx.x; k <= cg; k += TP_THREADS) gS[k] = gstart[g0 + k] - e0;
    for (int k = threadIdx.x; k < cg; k += TP_THREADS) cS[k] = gchild[g0 + k];
    for (int k = threadIdx.x; k < cg * 6; k += TP_THREADS) mS[k] = gmask[(int64_t) g0 * 6 + k];
    for (int32_t e = threadIdx.x; e < e1 - e0; e += TP_THREADS) fS[e] = f[e0 + e];
    __syncthreads();
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      for (int j = 0; j < cg; j++) {
        const uint32_t *mk = mS + j * 6;   // need[3], take[3]
        const unsigned ch = (unsigned) cS[j];
        for (int q = lane; q < NPE; q += 32) m[q] = ((mk[3 + (q >> 5)] >> (q & 31)) & 1u) ? prevS[q] : 0.0;
        __syncwarp();
#pragma unroll
        for (int ax = 0; ax < DIM; ax++) {
          const int s = ax == 0 ? 1 : (ax == 1 ? 3 : (ax == 2 ? 9 : 27));
          if (lane < NL) {
            const int base = (lane % s) + (lane / s) * 3 * s;
            double a = m[base], b = m[base + s], c = m[base + 2 * s];
            ip_line(a, b, c, pa, pb, pc, (ch >> ax) & 1u);
            m[base] = a;
            m[base + s] = b;
            m[base + 2 * s] = c;
          }
          __syncwarp();
        }
        const int ge = gS[j];
        for (int q = lane; q < NPE; q += 32) {
          const uint32_t w = mk[q >> 5];
          if ((w >> (q & 31)) & 1u) {
            int r = __popc(w & ((1u << (q & 31)) - 1u));   // rank among the needed slots
            for (int ww = 0; ww < (q >> 5); ww++) r += __popc(mk[ww]);
            const double val = fS[ge + r] + m[q];
            v[e0 + ge + r] = val;
            prevS[q] = val;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
    g0 += cg;
  }
  }
}

// Blocks of a chain launch: at most eight per SM, each taking runs in turn
// from the list (longest first).  One block per run would fill the SMs'
// block slots with short-lived chain blocks at the start of the product and
// hold back the leaf kernel it overlaps (level-8 moving ball: 3.93 ms for the
// leaf kernel beside a one-block-per-run chain, 3.76 ms beside four blocks
// per SM, with an earlier leaf kernel).  On the current leaf kernel the
// level-8 product does not depend on the chain's width (step 3.43 ms with
// two, four or eight blocks per SM), while on smaller meshes the chain is the
// longer of the two and more walkers shorten it (level 7: step 0.680 ms with
// two per SM, 0.630 with four, 0.598 with eight).
static unsigned chain_blocks(int64_t n_runs)
{
  int dev = 0, sms = 0;
  DKT_CUDA(cudaGetDevice(&dev));
  DKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  return (unsigned) std::max<int64_t>(1, std::min<int64_t>(n_runs, (int64_t) 8 * std::max(sms, 1)));
}

void stale_eval(Plan &pl, const double *x, const long long *xq, cudaStream_t s)
{
  if (!pl.st_ready || pl.st_n_runs == 0) return;
  const int64_t ne = pl.st_n_ent;
  const int npe = pl.npe;
  // small chunks keep the block's shared memory (~18 KB for Q1) low, so the
  // chain coexists with the tiled kernel it overlaps
  const int ch_t = std::max(1024, npe * npe);
  const size_t smem = (size_t) ch_t * 12 + (size_t) 2 * CH_E * 8 + (size_t) npe * 8 + (size_t) (CH_E + 1) * 4
                      + (size_t) (CH_G + 1) * 4 + 64;
  const unsigned blocks = chain_blocks(pl.st_n_runs);
  if (pl.st_tp) {
    if (xq) throw std::runtime_error("stale_eval: the order-2 walk has no fixed-point variant");
    k_stale_fresh<false><<<grid_for(ne, 256), 256, 0, s>>>(ne, pl.st_row.p, pl.st_idx.p, pl.st_w.p, x, nullptr,
                                                            pl.st_f.p);
    const double pa = pl.st_pint[0], pb = pl.st_pint[1], pc = pl.st_pint[2];
    switch (pl.dim) {
      case 2: k_stale_chain_tp<2><<<blocks, TP_THREADS, 0, s>>>(pl.st_runs.p, pl.st_n_runs, pl.st_gstart.p,
                                                                pl.st_gchild.p, pl.st_gmask.p, pl.st_f.p, pl.st_v.p,
                                                                pa, pb, pc); break;
      case 3: k_stale_chain_tp<3><<<blocks, TP_THREADS, 0, s>>>(pl.st_runs.p, pl.st_n_runs, pl.st_gstart.p,
                                                                pl.st_gchild.p, pl.st_gmask.p, pl.st_f.p, pl.st_v.p,
                                                                pa, pb, pc); break;
      default: k_stale_chain_tp<4><<<blocks, TP_THREADS, 0, s>>>(pl.st_runs.p, pl.st_n_runs, pl.st_gstart.p,
                                                                 pl.st_gchild.p, pl.st_gmask.p, pl.st_f.p, pl.st_v.p,
                                                                 pa, pb, pc); break;
    }
    check_launch("stale_eval_tp");
    pl.n_launch += 2;
    return;
  }
  if (xq) {
    k_stale_fresh<true><<<grid_for(ne, 256), 256, 0, s>>>(ne, pl.st_row.p, pl.st_idx.p, pl.st_w.p, nullptr, xq,
                                                           pl.st_f.p);
    auto kfn = k_stale_chain<true>;
    ensure_dyn_smem(kfn, smem);
    kfn<<<blocks, CH_THREADS, smem, s>>>(pl.st_runs.p, pl.st_n_runs, pl.st_gstart.p, pl.st_srow.p, pl.st_sidx.p,
                                         pl.st_sw.p, pl.st_f.p, pl.st_v.p, pl.st_vq.p, ch_t, npe);
  } else {
    k_stale_fresh<false><<<grid_for(ne, 256), 256, 0, s>>>(ne, pl.st_row.p, pl.st_idx.p, pl.st_w.p, x, nullptr,
                                                            pl.st_f.p);
    auto kfn = k_stale_chain<false>;
    ensure_dyn_smem(kfn, smem);
    kfn<<<blocks, CH_THREADS, smem, s>>>(pl.st_runs.p, pl.st_n_runs, pl.st_gstart.p, pl.st_srow.p, pl.st_sidx.p,
                                         pl.st_sw.p, pl.st_f.p, pl.st_v.p, nullptr, ch_t, npe);
  }
  check_launch("stale_eval");
  pl.n_launch += 2;
}

}  // namespace dkt
