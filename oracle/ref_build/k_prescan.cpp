// Reference kernel/preScan.cl compiled as C++ (TEST INFRASTRUCTURE ONLY).
#include "clc_prelude.hpp"
namespace refk_prescan {
#include "clc_builtins.hpp"
#include "preScan.cl"
}
extern "C" void refk_preScan(size_t gsize, void* states, void* pop, void* data, void* flags,
                             unsigned start, unsigned b1, unsigned b2, unsigned end, int match) {
  #pragma omp parallel for schedule(static)
  for (long g = 0; g < (long)gsize; g++) {
    clc_tls_gid = (size_t)g; clc_tls_gsize = gsize;
    refk_prescan::preScan((refk_prescan::AgentState*)states, (refk_prescan::Population*)pop, (int*)data,
                          (unsigned*)flags, start, b1, b2, end, match);
  }
}
