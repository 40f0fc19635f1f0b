/*
 * siminf_models_b.cu -- the kernel templates of siminf_kernels.cuh
 * instantiated for the shipped SISe models (plain, particle filter, spatial)
 * (siminf_models.cuh), in a unit of their own so that the model
 * instantiations compile in parallel.
 */
#include "siminf_kernels.cuh"

namespace siminf {

namespace {

struct Entry {
    const char *name;
    const Launchers *(*table)();
};

bool same_name(const char *a, const char *b)
{
    while (*a && *a == *b) {
        a++;
        b++;
    }
    return *a == 0 && *b == 0;
}

}  // namespace

const Launchers *launchers_shipped_b(const char *name)
{
    static const Entry entries[] = {
        {"SISe", Launch<ModelSISe>::table},
        {"SISe_pf", Launch<ModelSISePF>::table},
        {"SISe_sp", Launch<ModelSISe_sp>::table},
    };
    for (const Entry &e : entries)
        if (same_name(e.name, name))
            return e.table();
    return nullptr;
}

}  // namespace siminf
