// Host-side series set-up: delay schedule and q-partition mapping.
#include <cmath>
#include <map>
#include <set>

#include "xpcs_internal.h"

namespace xg {

// Corr::calculateLevelMax (src/xpcs/corr.cpp:1156-1160) and
// Corr::delaysPerLevel (src/xpcs/corr.cpp:1133-1154): level 0 holds 2*dpl
// delays of step 1, level i holds dpl delays of step 2^i, and a delay is kept
// while (previous delay) + 2^i + 2^i <= frames.  The same double-precision
// log2 expression decides the last level considered.
DelaySchedule delay_schedule(int frames, int dpl) {
  DelaySchedule d;
  if (frames <= 0 || dpl <= 0) return d;
  int max_level = 0;
  if (frames >= dpl * 2)
    max_level = (int)(std::floor(std::log2((double)frames) - std::log2(1.0 + 1.0 / (double)dpl)) -
                      std::log2((double)dpl));
  long long ll = 0;
  for (int i = 0; i <= max_level && i < 62; i++) {
    long long step = 1ll << i;
    int per_level = i == 0 ? 2 * dpl : dpl;
    for (int j = 0; j < per_level; j++) {
      if (ll + step + step > frames) break;
      d.level.push_back(i);
      d.tau.push_back((int32_t)(ll + step));
      ll += step;
    }
  }
  return d;
}

// Configuration::BuildQMap (src/xpcs/configuration.cpp:244-381), keeping the
// reference's observable behaviour:
//  * a pixel is valid when dqmap >= 1 and sqmap >= 1;
//  * the static-partition total only grows on pixels whose q was already
//    seen (:266-274), so it can undercount (quirk Q5);
//  * an sbin that appears under several q keeps only the q with the most
//    pixels (first in ascending q on ties); the reference's merge works on a
//    copy (:327-328), so that sbin's pixels under the other q are dropped
//    (quirk Q6) while the other q stay in the mapping;
//  * pixels_per_bin counts every valid pixel by its sbin.
// Maps the reference would index out of bounds are reported in `error`.
QMap build_qmap(const int32_t *dq, const int32_t *sq, int32_t pixels) {
  QMap m;
  m.pixels = pixels;
  m.valid.assign(pixels, 0);
  m.sbin.assign(pixels, 0);
  std::map<int, std::map<int, std::vector<int32_t>>> mapping;
  std::map<int, std::set<int>> sbin_to_q;
  for (int32_t i = 0; i < pixels; i++) {
    if (dq[i] < 1 || sq[i] < 1) continue;
    m.valid[i] = 1;
    m.sbin[i] = sq[i];
    if (m.total_dynamic < dq[i]) m.total_dynamic = dq[i];
    auto it = mapping.find(dq[i]);
    if (it != mapping.end()) {
      if (m.total_static < sq[i]) m.total_static = sq[i];
      it->second[sq[i]].push_back(i);
    } else {
      mapping[dq[i]][sq[i]].push_back(i);
    }
    sbin_to_q[sq[i]].insert(dq[i]);
  }
  for (auto &kv : sbin_to_q) {
    if (kv.second.size() < 2) continue;
    int sbin = kv.first, best_q = 0;
    size_t best_n = 0;
    for (int q : kv.second) {
      size_t n = mapping[q][sbin].size();
      if (n > best_n) {
        best_n = n;
        best_q = q;
      }
    }
    for (int q : kv.second)
      if (q != best_q) mapping[q].erase(sbin);
  }
  m.pixels_per_bin.assign(m.total_static > 0 ? m.total_static : 0, 0);
  for (int32_t i = 0; i < pixels; i++) {
    if (dq[i] < 1 || sq[i] < 1) continue;
    if (sq[i] > m.total_static) {
      m.error = "static partition " + std::to_string(sq[i]) +
                " exceeds the partition total the reference derives (" +
                std::to_string(m.total_static) + ")";
      continue;
    }
    m.pixels_per_bin[sq[i] - 1]++;
  }
  m.q_entry_ptr.push_back(0);
  m.entry_pix_ptr.push_back(0);
  const int nq = (int)mapping.size();
  for (auto &qv : mapping) {
    if (qv.first > nq && m.error.empty())
      m.error = "dynamic partition " + std::to_string(qv.first) +
                " exceeds the number of dynamic partitions in the map (" + std::to_string(nq) +
                ")";
    m.q_ids.push_back(qv.first);
    for (auto &sv : qv.second) {
      m.entry_sbin.push_back(sv.first);
      m.pix.insert(m.pix.end(), sv.second.begin(), sv.second.end());
      m.entry_pix_ptr.push_back((int32_t)m.pix.size());
    }
    m.q_entry_ptr.push_back((int32_t)m.entry_sbin.size());
  }
  return m;
}

}  // namespace xg
