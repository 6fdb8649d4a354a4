// Reference kernel/initAgents.cl compiled as C++ (TEST INFRASTRUCTURE ONLY).
#include "clc_prelude.hpp"
namespace refk_init {
#include "clc_builtins.hpp"
#include "initAgents.cl"
}
extern "C" void refk_initAgents(size_t gsize, void* agents, void* ages, void* states, void* enb, float T, void* seeds) {
  #pragma omp parallel for schedule(static)
  for (long g = 0; g < (long)gsize; g++) {
    clc_tls_gid = (size_t)g; clc_tls_gsize = gsize;
    refk_init::initAgents((refk_init::Agent*)agents, (refk_init::AgentAge*)ages, (refk_init::AgentState*)states,
                          (refk_init::EggsNbiomass*)enb, T, (refk_init::Seeds*)seeds);
  }
}
