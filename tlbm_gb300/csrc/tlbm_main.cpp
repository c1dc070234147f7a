// tlbm_main.cpp -- tLBMexec: the reference's driver (src/tLBM.cpp:7-88) over the C ABI.
//
// Run in a directory holding params.lbm, ndType.lbm and parts.lbm.  Prints the same progress,
// timing and "Estimated LPU/s" lines, dumps on (ts+1) % plotFreq == 0 && ts+1 > warmupTs and
// writes time averages when requested.  The wall-clock timer spans the whole step loop,
// dumps included, like the reference's MPI_Wtime pair.  Steps between two events (a progress
// line or a dump) are issued as CUDA graph launches.
//
//   tLBMexec [-np N] [--precision f64|f32|bf16|f16|bf16m] [--arithmetic reference|fast]
//            [--metrics FILE]
//   -np N           job size the parts.lbm file was made for (default: any partition ids)
//   --metrics FILE  also write the run's figures as one JSON object (nodes, steps, dumps,
//                   elapsed seconds, LPU/s, precision, arithmetic) to FILE
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "tlbm.h"

static int fail(tlbm_handle* h, tlbm_status s) {
  std::fprintf(stderr, "tLBMexec: %s: %s\n", tlbm_status_string(s), tlbm_get_last_error(h));
  if (h) tlbm_destroy(h);
  return 1;
}

int main(int argc, char* argv[]) {
  int size = INT_MAX / 2;
  bool have_opts = false;
  std::string metrics;
  tlbm_options opt;
  tlbm_default_options(&opt);
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "-np" && i + 1 < argc) {
      size = std::atoi(argv[++i]);
    } else if (a == "--precision" && i + 1 < argc) {
      std::string v = argv[++i];
      have_opts = true;
      if (v == "f64") opt.precision = TLBM_PREC_F64;
      else if (v == "f32") opt.precision = TLBM_PREC_F32;
      else if (v == "bf16") { opt.precision = TLBM_PREC_BF16; opt.arithmetic = TLBM_ARITH_FAST; }
      else if (v == "f16") { opt.precision = TLBM_PREC_F16; opt.arithmetic = TLBM_ARITH_FAST; }
      else if (v == "bf16m") { opt.precision = TLBM_PREC_BF16M; opt.arithmetic = TLBM_ARITH_FAST; }
      else { std::fprintf(stderr, "unknown precision %s\n", v.c_str()); return 2; }
    } else if (a == "--arithmetic" && i + 1 < argc) {
      std::string v = argv[++i];
      have_opts = true;
      opt.arithmetic = (v == "fast") ? TLBM_ARITH_FAST : TLBM_ARITH_REFERENCE;
    } else if (a == "--metrics" && i + 1 < argc) {
      metrics = argv[++i];
    } else {
      std::fprintf(stderr,
                   "usage: tLBMexec [-np N] [--precision P] [--arithmetic A] [--metrics FILE]\n");
      return 2;
    }
  }
  std::printf("Commencing test with %d processes\n", 1);
  tlbm_handle* h = nullptr;
  tlbm_status s = have_opts ? tlbm_create_ex(".", 0, size, &opt, &h) : tlbm_create(".", 0, size, &h);
  if (s != TLBM_OK) return fail(nullptr, s);

  const int num_ts = tlbm_get_num_ts(h);
  const int rep = tlbm_get_ts_rep_freq(h);
  const int warmup = tlbm_get_warmup_ts(h);
  const int plot = tlbm_get_plot_freq(h);
  const int time_avg = tlbm_get_time_avg_flag(h);

  int dumps = 0;
  auto t0 = std::chrono::steady_clock::now();
  int ts = 0;
  while (ts < num_ts) {
    // next step after which something happens on the host
    int stop = ts;
    while (stop < num_ts) {
      const int k = stop + 1;
      const bool report = rep > 0 && k % rep == 0;
      const bool dump = (k % plot == 0) && (k > warmup);
      if (report || dump) break;
      ++stop;
    }
    if (stop > ts) {
      if ((s = tlbm_run(h, ts, stop - ts)) != TLBM_OK) return fail(h, s);
      ts = stop;
      continue;
    }
    if (rep > 0 && (ts + 1) % rep == 0) std::printf("Executing time step: %d \n", ts + 1);
    if ((s = tlbm_step(h, ts % 2)) != TLBM_OK) return fail(h, s);
    if (((ts + 1) % plot == 0) && ((ts + 1) > warmup)) {
      if ((s = tlbm_write_data(h)) != TLBM_OK) return fail(h, s);
      ++dumps;
    }
    ++ts;
  }
  if ((s = tlbm_synchronize(h)) != TLBM_OK) return fail(h, s);
  const double exec_time =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("Test complete.\n");
  std::printf("Elapsed time: %g seconds \n", exec_time);
  const double nodes = static_cast<double>(tlbm_get_num_global_nodes(h));
  const double lpus = nodes * static_cast<double>(num_ts) / exec_time;
  std::printf("Estimated LPU/s = %g \n", lpus);
  if (!metrics.empty()) {
    static const char* kPrec[] = {"f64", "f32", "bf16", "f16", "bf16m"};
    tlbm_options run_opt;
    run_opt.struct_size = sizeof(run_opt);
    if ((s = tlbm_get_options(h, &run_opt)) != TLBM_OK) return fail(h, s);
    const int p = run_opt.precision >= 0 && run_opt.precision < 5 ? run_opt.precision : 1;
    FILE* m = std::fopen(metrics.c_str(), "w");
    if (!m) {
      std::fprintf(stderr, "tLBMexec: cannot write %s\n", metrics.c_str());
      tlbm_destroy(h);
      return 1;
    }
    std::fprintf(m,
                 "{\"nodes\": %.0f, \"steps\": %d, \"dumps\": %d, \"elapsed_s\": %.6f, "
                 "\"lpu_s\": %.6g, \"precision\": \"%s\", \"arithmetic\": \"%s\"}\n",
                 nodes, num_ts, dumps, exec_time, lpus, kPrec[p],
                 run_opt.arithmetic == TLBM_ARITH_FAST ? "fast" : "reference");
    std::fclose(m);
  }
  if (time_avg == 1) {
    std::printf("Writing time average data.\n");
    if ((s = tlbm_write_time_avg_data(h)) != TLBM_OK) return fail(h, s);
  }
  tlbm_destroy(h);
  return 0;
}
