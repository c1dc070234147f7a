// tLBM_main_over_abi.cpp -- the reference's driver (src/tLBM.cpp:7-88) rewritten over the C ABI
// of include/tlbm.h: the MPI calls go away and the time-step loop is unchanged.  Build:
//   g++ -std=c++17 -I include tlbm_gb300/examples/tLBM_main_over_abi.cpp \
//       -L tlbm_gb300/lib -ltlbm_gb300 -o tLBMexec
#include <cstdio>
#include <chrono>
#include "tlbm.h"          // was: #include <mpi.h> / "TLBM_Partition.h"

int main(int argc, char* argv[]) {
  printf("Commencing test with %d processes\n", 1);
  tlbm_handle* part = nullptr;
  if (tlbm_create(".", /*rank=*/0, /*size=*/1 << 20, &part) != TLBM_OK) {
    fprintf(stderr, "%s\n", tlbm_get_last_error(nullptr));
    return 1;
  }
  const int numTs = tlbm_get_num_ts(part), tsRepFreq = tlbm_get_ts_rep_freq(part);
  const int warmupTs = tlbm_get_warmup_ts(part), plotFreq = tlbm_get_plot_freq(part);
  auto t0 = std::chrono::steady_clock::now();
  for (int ts = 0; ts < numTs; ++ts) {
    if ((ts + 1) % tsRepFreq == 0) printf("Executing time step: %d \n", ts + 1);
    tlbm_step(part, ts % 2);                                   // take_LBM_time_step(ts%2)
    if (((ts + 1) % plotFreq == 0) & ((ts + 1) > warmupTs))
      tlbm_write_data(part);                                   // write_data()
  }
  tlbm_synchronize(part);
  double execTime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  printf("Test complete.\nElapsed time: %g seconds \n", execTime);
  printf("Estimated LPU/s = %g \n", double(tlbm_get_num_global_nodes(part)) * numTs / execTime);
  if (tlbm_get_time_avg_flag(part) == 1) tlbm_write_time_avg_data(part);
  tlbm_destroy(part);
}
