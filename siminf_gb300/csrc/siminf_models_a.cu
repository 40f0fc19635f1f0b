/*
 * siminf_models_a.cu -- the kernel templates of siminf_kernels.cuh
 * instantiated for the shipped SIR, SEIR, SIS and mparse SIR models
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

const Launchers *launchers_shipped_a(const char *name)
{
    static const Entry entries[] = {
        {"SIR", Launch<ModelSIR>::table},
        {"SEIR", Launch<ModelSEIR>::table},
        {"SIS", Launch<ModelSIS>::table},
        {"SIR_mparse", Launch<ModelSIRmparse>::table},
    };
    for (const Entry &e : entries)
        if (same_name(e.name, name))
            return e.table();
    return nullptr;
}

}  // namespace siminf
