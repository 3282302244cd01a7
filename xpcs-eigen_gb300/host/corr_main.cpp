// corr — the multi-tau XPCS driver on the GB300 library.
//
// Same command line and the same output datasets as xpcs-eigen's `corr`
// (src/xpcs/main.cpp:86-479): the analysis configuration (entry /xpcs by
// default) names the IMM frame file; the results are written into the same
// file under the configured output group:
//   pixelSum, frameSum, partition-mean-total, partition-mean-partial,
//   partition_norm_factor, timestamp_clock, timestamp_tick, then for the
//   multi-tau analysis tau, norm-0-g2, norm-0-stderr (and with --g2out
//   G2/IP/IF), for the two-time analysis (analysis_type Twotime) sg,
//   C2T_all/g2_<q>, g2full, g2partials; with --darkout DarkAvg/DarkStd.
// The analysis file is an HDF5 file (h5lite.h: the results are written into
// it, new datasets and groups appended, existing ones of the same type and
// shape overwritten, as H5Result does) or an XH5C container with the same
// paths (xh5c.h); the two are told apart by the file's signature.  Datasets
// are written contiguous, without the reference's optional deflate
// (h5_result.cpp:82-95): the values are the same, only the storage differs.
// Extra flags: --mode=exact (lookup over the live prefix only),
// --fp64 (write the float64 normalisation), --device=N, --block=N (frames
// per ingest call), --dry-run (read and check the configuration and every
// frame the analysis would use, report, and stop before any GPU work).
// Input errors the reference lets through -- a frame whose dlen exceeds the
// detector (sparse) or differs from it (dense), a pixel index outside the
// detector, a file that ends before the configured frames -- stop the run
// with a message and exit status 1.
#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "imm.h"
#include "xh5c.h"
#include "xpcs_gpu.h"

namespace {

struct Flags {
  bool g2out = false, darkout = false, fp64 = false, frame_threading = false, dry_run = false;
  int frameout = 0, device = 0, block = 512;
  std::string imm, inpath, outpath, exchange, entry, mode = "reference";
  std::vector<std::string> positional;
};

bool parse(int argc, char **argv, Flags &f, std::string &err) {
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    if (a.rfind("--", 0) != 0) {
      f.positional.push_back(a);
      continue;
    }
    std::string k = a.substr(2), v;
    bool has_v = false;
    size_t eq = k.find('=');
    if (eq != std::string::npos) {
      v = k.substr(eq + 1);
      k = k.substr(0, eq);
      has_v = true;
    }
    auto boolean = [&](bool &b) { b = !has_v || v == "true" || v == "1"; };
    if (k == "g2out") boolean(f.g2out);
    else if (k == "darkout") boolean(f.darkout);
    else if (k == "fp64") boolean(f.fp64);
    else if (k == "frameout") f.frameout = atoi(v.c_str());
    else if (k == "device") f.device = atoi(v.c_str());
    else if (k == "block") f.block = atoi(v.c_str());
    else if (k == "imm") f.imm = v;
    else if (k == "inpath") f.inpath = v;
    else if (k == "outpath") f.outpath = v;
    else if (k == "exchange") f.exchange = v;
    else if (k == "entry") f.entry = v;
    else if (k == "mode") f.mode = v;
    else if (k == "frame_threading") boolean(f.frame_threading);
    else if (k == "dry-run" || k == "dry_run") boolean(f.dry_run);
    else if (k == "ufxc" || k == "rigaku" || k == "hdf5" || k == "transposed") {
      err = "--" + k + " selects a reader or analysis outside the multi-tau IMM path";
      return false;
    } else {
      err = "unknown flag --" + k;
      return false;
    }
  }
  return true;
}

std::string lower(std::string s) {
  for (auto &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

struct Timer {
  const char *name;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit Timer(const char *n) : name(n) {}
  ~Timer() {
    double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                    .count();
    printf("[corr] %s took %.3f ms\n", name, ms);
  }
};

#define CHECK(call)                                                     \
  do {                                                                  \
    int rc_ = (call);                                                   \
    if (rc_ != XPCS_OK) {                                               \
      fprintf(stderr, "corr: %s failed (%d): %s\n", #call, rc_, xpcs_last_error()); \
      return 1;                                                         \
    }                                                                   \
  } while (0)

// The filter's side datasets (main.cpp:314-411): pixelSum, frameSum, the
// partition means, the normalisation factor and the timestamps.
int write_side(xh5c::File &cfg, xpcs_series *s, const std::string &g, int W, int H, int F,
               int swin, int S, float nf, const std::vector<double> &clock,
               const std::vector<double> &ticks, int real) {
  const int nwin = swin > 0 ? F / swin : 0;
  std::vector<float> psum((size_t)W * H), fsum(2 * (size_t)F), ptot(S), ppart((size_t)nwin * S);
  const int rc = xpcs_side_stats(s, psum.data(), fsum.data(), ptot.data(), ppart.data());
  if (rc != XPCS_OK) return rc;
  cfg.put(g + "pixelSum", xh5c::F32, {(uint64_t)H, (uint64_t)W}, psum.data());
  cfg.put(g + "frameSum", xh5c::F32, {2, (uint64_t)F}, fsum.data());
  cfg.put(g + "partition-mean-total", xh5c::F32, {1, (uint64_t)S}, ptot.data());
  cfg.put(g + "partition-mean-partial", xh5c::F32, {(uint64_t)nwin, (uint64_t)S}, ppart.data());
  cfg.put(g + "partition_norm_factor", xh5c::F32, {1, 1}, &nf);
  cfg.put(g + "timestamp_clock", xh5c::F64, {2, (uint64_t)real}, clock.data());
  cfg.put(g + "timestamp_tick", xh5c::F64, {2, (uint64_t)real}, ticks.data());
  return XPCS_OK;
}

}  // namespace

int main(int argc, char **argv) {
  Flags fl;
  std::string err;
  if (!parse(argc, argv, fl, err) || fl.positional.empty()) {
    fprintf(stderr, "%s\nusage: corr <analysis file> [--g2out] [--darkout] [--imm=path] "
            "[--inpath=a --outpath=b] [--exchange=group] [--entry=path] [--mode=exact] "
            "[--fp64] [--device=N]\n", err.empty() ? "Please specify a metadata file" : err.c_str());
    return 1;
  }
  Timer total("Total");
  const std::string cfg_path = fl.positional[0];
  const std::string entry = fl.entry.empty() ? "/xpcs" : fl.entry;
  xh5c::File cfg;
  if (!cfg.load(cfg_path)) {
    fprintf(stderr, "corr: cannot read %s%s%s\n", cfg_path.c_str(),
            cfg.error().empty() ? "" : ": ", cfg.error().c_str());
    return 1;
  }
  try {
    // Configuration::init (configuration.cpp:80-242)
    std::string output = cfg.get_string(entry + "/output_data");
    if (!fl.exchange.empty()) output = fl.exchange;
    int W = (int)cfg.get_scalar("/measurement/instrument/detector/x_dimension");
    int H = (int)cfg.get_scalar("/measurement/instrument/detector/y_dimension");
    std::vector<int32_t> dq = cfg.get_i32(entry + "/dqmap"), sq = cfg.get_i32(entry + "/sqmap");
    if (cfg.has(entry + "/transposed") && cfg.get_string(entry + "/transposed") == "ENABLED") {
      std::vector<int32_t> d2(dq.size()), s2(sq.size());
      for (int i = 0; i < W * H; i++) {
        int row = i % W, col = i / W, idx = row * H + col;
        d2[idx] = dq[i];
        s2[idx] = sq[i];
      }
      dq.swap(d2);
      sq.swap(s2);
      std::swap(W, H);
    }
    const int begin_todo = (int)cfg.get_scalar(entry + "/data_begin_todo");
    const int end_todo = (int)cfg.get_scalar(entry + "/data_end_todo");
    const int dpl = (int)cfg.get_scalar(entry + "/delays_per_level");
    int dark_b = (int)cfg.get_scalar(entry + "/dark_begin_todo");
    int dark_e = (int)cfg.get_scalar(entry + "/dark_end_todo");
    const int stride = (int)cfg.get_scalar(entry + "/stride_frames");
    const int avg = (int)cfg.get_scalar(entry + "/avg_frames");
    const int swin = (int)cfg.get_scalar(entry + "/static_mean_window_size");
    const bool by_framesum = cfg.has(entry + "/normalize_by_framesum") &&
                             cfg.get_scalar(entry + "/normalize_by_framesum") != 0;
    // two-time options (configuration.cpp:150-151, 216-231; main.cpp:161-164)
    const bool twotime = cfg.has(entry + "/analysis_type") &&
                         cfg.get_string(entry + "/analysis_type") == "Twotime";
    xpcs_twotime_desc tdesc{};
    std::vector<int32_t> tq;
    if (twotime) {
      const std::string method = lower(cfg.get_string(entry + "/smoothing_method"));
      if (method != "staticmap" && method != "symmetric") {
        fprintf(stderr, "Smoothing method is not valid\n");
        return 1;
      }
      tdesc.static_map = method == "staticmap";
      tdesc.average = lower(cfg.get_string(entry + "/smoothing_filter")) == "average";
      for (double q : cfg.get_f64(entry + "/qphi_bin_to_process")) tq.push_back((int32_t)q);
      tdesc.qbins = tq.data();
      tdesc.nqbins = (int32_t)tq.size();
      tdesc.window = cfg.has(entry + "/twotime2onetime_window_size")
                         ? (int32_t)cfg.get_scalar(entry + "/twotime2onetime_window_size")
                         : 1;
      tdesc.frame_threading = fl.frame_threading;
    }
    int darks = 0;
    float lld = 0.f, sigma = 0.f;
    if (!(dark_b == dark_e || dark_e == 0)) {
      darks = dark_e - dark_b + 1;
      lld = (float)cfg.get_scalar(entry + "/lld");
      sigma = (float)cfg.get_scalar(entry + "/sigma");
    }
    // the normalisation factor, float arithmetic as configuration.cpp:193-199
    const std::string det = "/measurement/instrument/detector/";
    float dpx = (float)cfg.get_scalar(det + "x_pixel_size");
    float dpy = (float)cfg.get_scalar(det + "y_pixel_size");
    float adu = (float)cfg.get_scalar(det + "adu_per_photon");
    float preset = (float)cfg.get_scalar(det + "exposure_time");
    float eff = (float)cfg.get_scalar(det + "efficiency");
    float dist = (float)cfg.get_scalar(det + "distance");
    float flux = (float)cfg.get_scalar("/measurement/instrument/source_begin/beam_intensity_transmitted");
    float thick = (float)cfg.get_scalar("/measurement/sample/thickness");
    volatile float nf = 1.0f;
    nf = nf / eff / adu / preset;
    volatile float geo = dpx / dist;
    geo = geo * dpy;
    geo = geo / dist;
    nf = nf / geo;
    nf /= flux;
    nf /= thick;
    std::vector<double> flat;
    const bool flat_on = cfg.get_string(entry + "/flatfield_enabled") == "ENABLED";
    if (flat_on) flat = cfg.get_f64(det + "flatfield");
    std::string imm_path = fl.imm.empty() ? cfg.get_string(entry + "/input_file_local") : fl.imm;
    if (!fl.inpath.empty() && !fl.outpath.empty()) {
      size_t pos = imm_path.find(fl.inpath);
      if (pos != std::string::npos) imm_path.replace(pos, fl.inpath.size(), fl.outpath);
    }
    const int real = end_todo - begin_todo + 1;
    const int F = real / (stride * avg);
    const int frame_from = begin_todo - 1;
    const int read_in = stride * avg;

    imm::Reader rd;
    if (!rd.open(imm_path)) {
      fprintf(stderr, "corr: cannot open IMM file %s\n", imm_path.c_str());
      return 1;
    }
    rd.set_frame_pixels((int64_t)W * H);
    printf("[corr] %s: %dx%d, %d frames (stride %d, average %d), %s frames\n", imm_path.c_str(),
           W, H, F, stride, avg, rd.compressed() ? "sparse" : "dense");
    if (dq.size() != (size_t)W * H || sq.size() != (size_t)W * H)
      throw std::runtime_error("dqmap/sqmap size differs from the detector's x_dimension * "
                               "y_dimension");
    if (flat_on && flat.size() != (size_t)W * H)
      throw std::runtime_error("flatfield size differs from the detector's pixel count");
    if (fl.dry_run) {
      // every frame the analysis would read, checked on the host; no GPU work
      imm::Block blk;
      int64_t r = 0, events = 0, bad = 0;
      if (!rd.compressed() && darks > 0) {
        const int n = rd.next(darks, blk);
        if (n < 0) throw std::runtime_error(rd.error());
        if (n != darks) throw std::runtime_error("short IMM file (darks)");
        r += darks;
      }
      if (frame_from > 0 && r < frame_from) {
        const int n = rd.skip((int)(frame_from - r));
        if (n < 0) throw std::runtime_error(rd.error());
        r += n;
      }
      const int64_t want = (int64_t)F * read_in;
      int64_t got = 0;
      while (got < want) {
        const int n = rd.next((int)std::min<int64_t>(fl.block, want - got), blk);
        if (n < 0) throw std::runtime_error(rd.error());
        if (n == 0) break;
        for (int32_t p : blk.idx) bad += (p < 0 || (int64_t)p >= (int64_t)W * H);
        events += (int64_t)blk.val.size();
        got += n;
      }
      if (got < want)
        throw std::runtime_error("IMM file ends after " + std::to_string(got) + " of " +
                                 std::to_string(want) + " frames");
      if (bad)
        throw std::runtime_error(std::to_string(bad) +
                                 " pixel indices lie outside the detector");
      int32_t nd = 0;
      CHECK(xpcs_delay_schedule(F, dpl, nullptr, nullptr, 0, &nd));
      printf("[corr] dry run: %d frames, %lld events, %d delays: input is valid\n", F,
             (long long)events, nd);
      return 0;
    }
    xpcs_series_desc d{};
    d.width = W;
    d.height = H;
    d.frames = F;
    d.delays_per_level = dpl;
    d.stride_frames = stride;
    d.avg_frames = avg;
    d.static_window = swin;
    d.dqmap = dq.data();
    d.sqmap = sq.data();
    d.flatfield = flat_on ? flat.data() : nullptr;
    d.dense = rd.compressed() ? 0 : 1;
    d.lld = lld;
    d.sigma = sigma;
    d.device = fl.device;
    d.normalize_by_framesum = by_framesum ? 1 : 0;
    xpcs_series *s = nullptr;
    CHECK(xpcs_series_create(&d, &s));
    xpcs_series_info info{};
    CHECK(xpcs_series_get_info(s, &info));
    const int P = info.pixels, D = info.delays, Q = info.qbins, S = info.total_static;

    std::vector<double> clock(2 * (size_t)real, 0.0), ticks(2 * (size_t)real, 0.0);
    {
      Timer t("Loading data");
      imm::Block blk;
      int r = 0;
      if (!rd.compressed() && darks > 0) {  // the first frames of the file (main.cpp:227-239)
        const int n = rd.next(darks, blk);
        if (n < 0) throw std::runtime_error(rd.error());
        if (n != darks) throw std::runtime_error("short IMM file (darks)");
        CHECK(xpcs_set_dark(s, blk.val.data(), darks));
        r += darks;
      }
      if (frame_from > 0 && r < frame_from) {
        const int n = rd.skip(frame_from - r);
        if (n < 0) throw std::runtime_error(rd.error());
        r += n;
      }
      const int want = F * read_in;
      int got = 0;
      while (got < want) {
        int n = rd.next(std::min(fl.block, want - got), blk);
        if (n < 0) throw std::runtime_error(rd.error());
        if (n == 0) break;
        if (rd.compressed())
          CHECK(xpcs_ingest_sparse(s, blk.idx.data(), blk.val.data(), blk.nnz.data(), n));
        else
          CHECK(xpcs_ingest_dense(s, blk.val.data(), n));
        for (int k = 0; k < n; k++) {
          const int g = got + k;
          clock[g] = g + 1;
          clock[g + real] = blk.clock[k];
          ticks[g] = g + 1;
          ticks[g + real] = blk.ticks[k];
        }
        got += n;
      }
      if (got < want)
        throw std::runtime_error("IMM file ends after " + std::to_string(got) + " of " +
                                 std::to_string(want) + " frames");
    }
    const std::string g = output + "/";
    if (twotime) {
      xpcs_twotime_info ti{};
      {
        Timer t("Computing G2 TwoTimes");
        CHECK(xpcs_twotime(s, &tdesc, XPCS_MODE_REFERENCE, &ti));
      }
      CHECK(write_side(cfg, s, g, W, H, F, swin, S, nf, clock, ticks, real));
      const uint64_t NQ = (uint64_t)ti.qbins, FF = (uint64_t)ti.frames;
      std::vector<int32_t> qs(NQ);
      std::vector<float> sg((size_t)ti.sg_rows * ti.sg_cols), c2t(NQ * FF * FF), full(FF * NQ),
          part((size_t)ti.window * ti.partials * NQ);
      CHECK(xpcs_get_twotime(s, qs.data(), sg.data(), c2t.data(), full.data(), part.data()));
      cfg.put(g + "sg", xh5c::F32, {(uint64_t)ti.sg_rows, (uint64_t)ti.sg_cols}, sg.data());
      for (uint64_t i = 0; i < NQ; i++) {
        char name[32];
        snprintf(name, sizeof(name), "g2_%05d", qs[i]);
        cfg.put(g + "C2T_all/" + name, xh5c::F32, {FF, FF}, c2t.data() + i * FF * FF);
      }
      cfg.put(g + "g2full", xh5c::F32, {FF, NQ}, full.data());
      cfg.put(g + "g2partials", xh5c::F32, {(uint64_t)ti.window, (uint64_t)ti.partials, NQ},
              part.data());
    } else {
      {
        Timer t("Computing G2 MultiTau");
        CHECK(xpcs_multitau(s, fl.mode == "exact" ? XPCS_MODE_EXACT : XPCS_MODE_REFERENCE));
        CHECK(xpcs_synchronize(s));
      }
      CHECK(write_side(cfg, s, g, W, H, F, swin, S, nf, clock, ticks, real));
      std::vector<int32_t> lv(D), tau(D);
      int32_t nd = 0;
      CHECK(xpcs_delay_schedule(F, dpl, lv.data(), tau.data(), D, &nd));
      std::vector<float> tauf(D);
      for (int k = 0; k < D; k++) tauf[k] = (float)tau[k];
      cfg.put(g + "tau", xh5c::F32, {1, (uint64_t)D}, tauf.data());
      Timer t("Normalizing Data");
      std::vector<double> g2d((size_t)D * Q), sed((size_t)D * Q);
      std::vector<float> g2f((size_t)D * Q), sef((size_t)D * Q);
      if (fl.fp64) {
        CHECK(xpcs_normalize(s, g2d.data(), sed.data(), nullptr, nullptr));
        for (size_t k = 0; k < g2f.size(); k++) {
          g2f[k] = (float)g2d[k];
          sef[k] = (float)sed[k];
        }
      } else {
        CHECK(xpcs_normalize(s, nullptr, nullptr, g2f.data(), sef.data()));
      }
      cfg.put(g + "norm-0-g2", xh5c::F32, {(uint64_t)D, (uint64_t)Q}, g2f.data());
      cfg.put(g + "norm-0-stderr", xh5c::F32, {(uint64_t)D, (uint64_t)Q}, sef.data());
      if (fl.g2out) {
        Timer t2("Writing G2s, IPs and IFs");
        std::vector<float> G2((size_t)D * P), IP(G2.size()), IF(G2.size());
        CHECK(xpcs_get_g2ipif(s, G2.data(), IP.data(), IF.data()));
        cfg.put(g + "G2", xh5c::F32, {(uint64_t)D, (uint64_t)P}, G2.data());
        cfg.put(g + "IP", xh5c::F32, {(uint64_t)D, (uint64_t)P}, IP.data());
        cfg.put(g + "IF", xh5c::F32, {(uint64_t)D, (uint64_t)P}, IF.data());
      }
    }
    if (!rd.compressed() && fl.darkout && darks > 0) {
      std::vector<double> da(P), ds(P);
      CHECK(xpcs_get_dark(s, da.data(), ds.data()));
      cfg.put(g + "DarkAvg", xh5c::F64, {(uint64_t)H, (uint64_t)W}, da.data());
      cfg.put(g + "DarkStd", xh5c::F64, {(uint64_t)H, (uint64_t)W}, ds.data());
    }
    xpcs_stage_times st{};
    xpcs_get_stage_times(s, &st);
    printf("[corr] GPU stages: filter %.3f ms, multi-tau %.3f ms, normalise %.3f ms\n",
           st.filter_ms, st.multitau_ms, st.normalize_ms);
    xpcs_series_destroy(s);
    if (!cfg.save(cfg_path)) {
      fprintf(stderr, "corr: cannot write %s%s%s\n", cfg_path.c_str(),
              cfg.error().empty() ? "" : ": ", cfg.error().c_str());
      return 1;
    }
  } catch (const std::exception &e) {
    fprintf(stderr, "corr: %s\n", e.what());
    return 1;
  }
  return 0;
}
