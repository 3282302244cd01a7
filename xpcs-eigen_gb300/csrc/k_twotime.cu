// F3: two-time correlation C2T(t1, t2) per q bin, with the reference's
// smoothing and its one-time reductions g2full / g2partials.
//
// Replaces Corr::twotime (src/xpcs/corr.cpp:560-924) with SmoothingStaticMap /
// SmoothingSymmetric (:433-547) and ComputeSG* (:1166-1305).  REFERENCE mode
// reproduces the reference's float32 operations in its order:
//   - the pixels of the processed q bins become rows of a dense matrix
//     V [rows][F] in mapping order (q, static bin, pixel), zero where a pixel
//     has no event;
//   - sg[g][f] = the float sum over the rows of smoothing group g (a static
//     bin, or a q bin for the symmetric method) in mapping order, / pixels;
//     with the average filter, the float mean over frames;
//   - every event value is divided by its sg;
//   - C_q[f0][f1] (f0 <= f1) = the float sum over the q bin's rows, in
//     mapping order (ascending pixel index with frame threading), of
//     v(f0) * v(f1) over pairs of events, then / pixels: a tiled CUDA-core
//     Gram whose reduction runs over the rows in order, one separate multiply
//     and add per pair (no fused multiply-add), products with a missing event
//     skipped as the reference never forms them;
//   - g2full[ff] = the float mean of diagonal ff in order; g2partials[ff][w]
//     the float sum of window w (`window` entries) of diagonal ff / window.
#include <algorithm>
#include <numeric>

#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int TT_TILE = 64;  // Gram tile (frames x frames)
constexpr int TT_KC = 32;    // rows per shared-memory chunk

__global__ void k_tt_scatter(int32_t R, int32_t F, const int32_t *__restrict__ row_pix,
                             const int64_t *__restrict__ row_ptr,
                             const int32_t *__restrict__ row_len,
                             const int32_t *__restrict__ ev_frame,
                             const float *__restrict__ ev_val, float *__restrict__ V) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int p = row_pix[r];
  const int64_t b = row_ptr[p];
  const int n = row_len[p];
  for (int i = 0; i < n; i++) {
    const int f = ev_frame[b + i];
    if (f >= 0 && f < F) V[(size_t)r * F + f] = ev_val[b + i];
  }
}

// sg[g][f]: float sum over the group's rows in order, / pixels
__global__ void k_tt_sg(int32_t G, int32_t F, const int32_t *__restrict__ grp_ptr,
                        const float *__restrict__ V, float *__restrict__ sg) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y;
  if (f >= F || g >= G) return;
  float acc = 0.f;
  for (int r = grp_ptr[g]; r < grp_ptr[g + 1]; r++) acc = __fadd_rn(acc, V[(size_t)r * F + f]);
  sg[(size_t)g * F + f] = __fdiv_rn(acc, (float)(grp_ptr[g + 1] - grp_ptr[g]));
}

__global__ void k_tt_sg_avg(int32_t G, int32_t F, const float *__restrict__ sg,
                            float *__restrict__ sga) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  float acc = 0.f;
  for (int f = 0; f < F; f++) acc = __fadd_rn(acc, sg[(size_t)g * F + f]);
  sga[g] = __fdiv_rn(acc, (float)F);
}

__global__ void k_tt_smooth(int32_t R, int32_t F, int32_t average,
                            const int32_t *__restrict__ row_grp, const float *__restrict__ sg,
                            float *__restrict__ V) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)R * F) return;
  const int r = (int)(i / F), f = (int)(i % F);
  const float v = V[i];
  if (v == 0.f) return;  // no event
  const int g = row_grp[r];
  V[i] = __fdiv_rn(v, average ? sg[g] : sg[(size_t)g * F + f]);
}

// One block per upper-triangle 64x64 tile of one q bin; 256 threads x 4x4 cells.
__global__ void __launch_bounds__(256)
k_tt_gram(int32_t F, int32_t nrows, const int32_t *__restrict__ order,
          const float *__restrict__ V, float *__restrict__ C) {
  __shared__ float As[TT_KC][TT_TILE];
  __shared__ float Bs[TT_KC][TT_TILE];
  // linear block id -> (bi <= bj)
  const int T = (F + TT_TILE - 1) / TT_TILE;
  int id = blockIdx.x, bi = 0;
  while (id >= T - bi) {
    id -= T - bi;
    bi++;
  }
  const int bj = bi + id;
  const int f0 = bi * TT_TILE, f1 = bj * TT_TILE;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < nrows; k0 += TT_KC) {
    for (int e = threadIdx.x; e < TT_KC * TT_TILE; e += 256) {
      const int kk = e / TT_TILE, c = e % TT_TILE;
      const bool in = k0 + kk < nrows;
      const size_t row = in ? (size_t)order[k0 + kk] * F : 0;
      As[kk][c] = (in && f0 + c < F) ? V[row + f0 + c] : 0.f;
      Bs[kk][c] = (in && f1 + c < F) ? V[row + f1 + c] : 0.f;
    }
    __syncthreads();
    const int kn = min(TT_KC, nrows - k0);
    for (int kk = 0; kk < kn; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const float pr = __fmul_rn(a[i], b[j]);
          acc[i][j] = (a[i] != 0.f && b[j] != 0.f) ? __fadd_rn(acc[i][j], pr) : acc[i][j];
        }
    }
    __syncthreads();
  }
  const float den = (float)nrows;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int r = f0 + ty * 4 + i, c = f1 + tx * 4 + j;
      if (r < F && c < F && r <= c) C[(size_t)r * F + c] = __fdiv_rn(acc[i][j], den);
    }
}

// one thread per (q, diagonal ff): g2full and, for ff < window, g2partials
__global__ void k_tt_diag(int32_t Q, int32_t F, int32_t window, int32_t tp,
                          const float *__restrict__ C, float *__restrict__ g2full,
                          float *__restrict__ g2part) {
  const int ff = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
  if (ff >= F || q >= Q) return;
  const float *Cq = C + (size_t)q * F * F;
  float acc = 0.f;
  for (int fx = 0; fx < F - ff; fx++) acc = __fadd_rn(acc, Cq[(size_t)fx * F + fx + ff]);
  g2full[(size_t)ff * Q + q] = __fdiv_rn(acc, (float)(F - ff));
  if (ff < window) {
    for (int w = 0; w < tp; w++) {
      float s = 0.f;
      for (int fx = w * window; fx < (w + 1) * window && fx < F - ff; fx++)
        s = __fadd_rn(s, Cq[(size_t)fx * F + fx + ff]);
      g2part[((size_t)ff * tp + w) * Q + q] = __fdiv_rn(s, (float)window);
    }
  }
}

}  // namespace

void run_twotime(Series &s, const TwoTimeReq &req, int mode, bool force_i64) {
  cudaStream_t st = s.stream;
  const QMap &qm = s.qmap;
  const int32_t F = s.F;
  TwoTimeOut &o = s.tt;
  o = TwoTimeOut{};
  o.frames = F;
  o.window = req.window;
  o.partials = req.window > 0 ? std::max(0, (F - req.window) / req.window) : 0;
  // rows of the processed q bins in mapping order; smoothing groups; q row ranges
  TwoTimeLayout lay;
  for (int32_t i = 0; i < qm.nq(); i++) {
    const int32_t q = qm.q_ids[i];
    if (std::find(req.qbins.begin(), req.qbins.end(), q) == req.qbins.end()) continue;
    for (int32_t e = qm.q_entry_ptr[i]; e < qm.q_entry_ptr[i + 1]; e++) {
      for (int32_t k = qm.entry_pix_ptr[e]; k < qm.entry_pix_ptr[e + 1]; k++) {
        lay.row_pix.push_back(qm.pix[k]);
        lay.row_grp.push_back((int32_t)lay.grp_ptr.size() - 1);
      }
      if (req.static_map) lay.grp_ptr.push_back((int32_t)lay.row_pix.size());
    }
    if (!req.static_map) lay.grp_ptr.push_back((int32_t)lay.row_pix.size());
    lay.q_ptr.push_back((int32_t)lay.row_pix.size());
    lay.q_grp_end.push_back((int32_t)lay.grp_ptr.size() - 1);
    o.qbins.push_back(q);
  }
  const std::vector<int32_t> &row_pix = lay.row_pix, &row_grp = lay.row_grp,
                             &grp_ptr = lay.grp_ptr, &q_ptr = lay.q_ptr;
  const int32_t R = (int32_t)row_pix.size(), G = (int32_t)grp_ptr.size() - 1,
                Q = (int32_t)o.qbins.size();
  o.sg_rows = G;
  o.sg_cols = req.average ? 1 : F;
  auto up = [&](DBuf<int32_t> &b, const std::vector<int32_t> &v) {
    b.reserve(v.size() ? v.size() : 1, st);
    if (!v.empty())
      XG_CUDA(cudaMemcpyAsync(b.p, v.data(), 4 * v.size(), cudaMemcpyHostToDevice, st));
  };
  up(s.tt_row_pix, row_pix);
  s.tt_sg.reserve((size_t)(G ? G : 1) * (F ? F : 1), st);
  s.tt_sga.reserve(G ? G : 1, st);
  s.tt_C.reserve((size_t)(Q ? Q : 1) * F * F + 1, st);
  s.tt_full.reserve((size_t)F * (Q ? Q : 1) + 1, st);
  s.tt_part.reserve((size_t)req.window * o.partials * (Q ? Q : 1) + 1, st);
  XG_CUDA(cudaMemsetAsync(s.tt_C.p, 0, 4 * ((size_t)Q * F * F + 1), st));
  if (mode == XPCS_MODE_EXACT) {
    if (R > 0 && F > 0) run_twotime_exact(s, req, lay, force_i64);
    o.ready = true;
    return;
  }
  // Gram order of every q bin's rows
  std::vector<int32_t> order(R);
  std::iota(order.begin(), order.end(), 0);
  if (req.frame_threading)
    for (int32_t q = 0; q < Q; q++)
      std::sort(order.begin() + q_ptr[q], order.begin() + q_ptr[q + 1],
                [&](int32_t a, int32_t b) { return row_pix[a] < row_pix[b]; });
  up(s.tt_row_grp, row_grp);
  up(s.tt_grp_ptr, grp_ptr);
  up(s.tt_order, order);
  const size_t nV = (size_t)R * F;
  s.tt_V.reserve(nV ? nV : 1, st);
  if (nV) XG_CUDA(cudaMemsetAsync(s.tt_V.p, 0, 4 * nV, st));
  if (R > 0 && F > 0) {
    k_tt_scatter<<<(R + 127) / 128, 128, 0, st>>>(R, F, s.tt_row_pix.p, s.row_ptr.p, s.row_len.p,
                                                  s.ev_frame.p, s.ev_val.p, s.tt_V.p);
    XG_CHECK_LAUNCH();
    k_tt_sg<<<dim3((F + 127) / 128, G), 128, 0, st>>>(G, F, s.tt_grp_ptr.p, s.tt_V.p, s.tt_sg.p);
    XG_CHECK_LAUNCH();
    if (req.average) {
      k_tt_sg_avg<<<(G + 127) / 128, 128, 0, st>>>(G, F, s.tt_sg.p, s.tt_sga.p);
      XG_CHECK_LAUNCH();
    }
    k_tt_smooth<<<(unsigned)((nV + 255) / 256), 256, 0, st>>>(R, F, req.average, s.tt_row_grp.p,
                                                             req.average ? s.tt_sga.p : s.tt_sg.p,
                                                             s.tt_V.p);
    XG_CHECK_LAUNCH();
    const int T = (F + TT_TILE - 1) / TT_TILE;
    for (int32_t q = 0; q < Q; q++) {
      const int32_t nr = q_ptr[q + 1] - q_ptr[q];
      if (nr == 0) continue;
      k_tt_gram<<<T * (T + 1) / 2, 256, 0, st>>>(F, nr, s.tt_order.p + q_ptr[q], s.tt_V.p,
                                                 s.tt_C.p + (size_t)q * F * F);
      XG_CHECK_LAUNCH();
    }
    k_tt_diag<<<dim3((F + 127) / 128, Q), 128, 0, st>>>(Q, F, req.window, o.partials, s.tt_C.p,
                                                       s.tt_full.p, s.tt_part.p);
    XG_CHECK_LAUNCH();
  }
  o.ready = true;
}

void get_twotime(Series &s, int32_t *qbins, float *sg, float *c2t, float *g2full,
                 float *g2part) {
  cudaStream_t st = s.stream;
  const TwoTimeOut &o = s.tt;
  const size_t Q = o.qbins.size(), F = (size_t)o.frames;
  if (qbins) std::copy(o.qbins.begin(), o.qbins.end(), qbins);
  if (sg && o.sg_rows)
    XG_CUDA(cudaMemcpyAsync(sg, o.sg_cols == 1 ? s.tt_sga.p : s.tt_sg.p,
                            4 * (size_t)o.sg_rows * o.sg_cols, cudaMemcpyDeviceToHost, st));
  if (c2t && Q) XG_CUDA(cudaMemcpyAsync(c2t, s.tt_C.p, 4 * Q * F * F, cudaMemcpyDeviceToHost, st));
  if (g2full && Q) XG_CUDA(cudaMemcpyAsync(g2full, s.tt_full.p, 4 * F * Q, cudaMemcpyDeviceToHost, st));
  if (g2part && Q && o.partials)
    XG_CUDA(cudaMemcpyAsync(g2part, s.tt_part.p, 4 * (size_t)o.window * o.partials * Q,
                            cudaMemcpyDeviceToHost, st));
  XG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace xg
