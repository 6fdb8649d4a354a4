// Reference kernel/oldToNewAgents.cl compiled as C++ (TEST INFRASTRUCTURE ONLY).
#include "clc_prelude.hpp"
namespace refk_o2n {
#include "clc_builtins.hpp"
#include "oldToNewAgents.cl"
}
extern "C" void refk_oldToNewAgents(size_t gsize, void* a, void* aa, void* as, void* na, void* naa, void* nas,
                                    void* p1, void* p2, void* p3, void* pop, void* enb) {
  #pragma omp parallel for schedule(static)
  for (long g = 0; g < (long)gsize; g++) {
    clc_tls_gid = (size_t)g; clc_tls_gsize = gsize;
    refk_o2n::oldToNewAgents((refk_o2n::Agent*)a, (refk_o2n::AgentAge*)aa, (refk_o2n::AgentState*)as,
                             (refk_o2n::Agent*)na, (refk_o2n::AgentAge*)naa, (refk_o2n::AgentState*)nas,
                             (int*)p1, (int*)p2, (int*)p3, (refk_o2n::Population*)pop, (refk_o2n::EggsNbiomass*)enb);
  }
}
