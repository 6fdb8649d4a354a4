// Reference kernel/ageHistogram.cl compiled as C++ (TEST INFRASTRUCTURE ONLY).
#include "clc_prelude.hpp"
namespace refk_hist {
#include "clc_builtins.hpp"
#include "ageHistogram.cl"
}
extern "C" void refk_ageHistogram(size_t gsize, void* ages, void* pop, void* hist) {
  #pragma omp parallel for schedule(static)
  for (long g = 0; g < (long)gsize; g++) {
    clc_tls_gid = (size_t)g; clc_tls_gsize = gsize;
    refk_hist::ageHistogram((refk_hist::AgentAge*)ages, (refk_hist::Population*)pop, (unsigned*)hist);
  }
}
