// tc_generate: the synthetic workloads of gen_core.h behind the C ABI.
#include "gen_core.h"
#include "timesc.h"

extern "C" int tc_generate(const tc_gen_spec* sp, float* data, int32_t* labels) {
    if (!sp) return TC_ERR_ARG;
    const tcgen::Params p{sp->n, sp->m, sp->classes, sp->noise, sp->dirichlet, sp->seed};
    return tcgen::generate(&p, data, labels) ? TC_OK : TC_ERR_ARG;
}
