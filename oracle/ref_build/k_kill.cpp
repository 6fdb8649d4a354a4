// Reference kernel/killAgents.cl compiled as C++ (TEST INFRASTRUCTURE ONLY).
#include "clc_prelude.hpp"
namespace refk_kill {
#include "clc_builtins.hpp"
#include "killAgents.cl"
}
extern "C" void refk_killAgents(size_t gsize, void* ages, void* states, void* pop, void* enb, void* bnc, void* seeds, float cc) {
  // gid 0 writes the per-step counters; run it alone before the others.
  clc_tls_gid = 0; clc_tls_gsize = gsize;
  refk_kill::killAgents((refk_kill::AgentAge*)ages, (refk_kill::AgentState*)states, (refk_kill::Population*)pop,
                        (refk_kill::EggsNbiomass*)enb, (refk_kill::BitesNcycles*)bnc, (refk_kill::Seeds*)seeds, cc);
  #pragma omp parallel for schedule(static)
  for (long g = 1; g < (long)gsize; g++) {
    clc_tls_gid = (size_t)g; clc_tls_gsize = gsize;
    refk_kill::killAgents((refk_kill::AgentAge*)ages, (refk_kill::AgentState*)states, (refk_kill::Population*)pop,
                          (refk_kill::EggsNbiomass*)enb, (refk_kill::BitesNcycles*)bnc, (refk_kill::Seeds*)seeds, cc);
  }
}
