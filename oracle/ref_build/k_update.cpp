// Reference kernel/updateAgents.cl (+ the species header) compiled as C++ (TEST INFRASTRUCTURE ONLY).
#include "clc_prelude.hpp"
namespace refk_update {
#include "clc_builtins.hpp"
#include "updateAgents.cl"
}
extern "C" void refk_updateAgents(size_t gsize, void* agents, void* ages, void* states, void* pop, const void* env,
                                  float T, void* bnc, void* enb, void* seeds, float dt, unsigned worldTime) {
  refk_update::Environment e;
  memcpy(&e, env, sizeof(e));
  #pragma omp parallel for schedule(static)
  for (long g = 0; g < (long)gsize; g++) {
    clc_tls_gid = (size_t)g; clc_tls_gsize = gsize;
    refk_update::updateAgents((refk_update::Agent*)agents, (refk_update::AgentAge*)ages, (refk_update::AgentState*)states,
                              (refk_update::Population*)pop, e, T, (refk_update::BitesNcycles*)bnc,
                              (refk_update::EggsNbiomass*)enb, (refk_update::Seeds*)seeds, dt, worldTime);
  }
}
extern "C" size_t refk_environment_size(void) { return sizeof(refk_update::Environment); }
