// relax_probe.cu -- batched LMO calls and node-feasibility checks.
#include "relax_impl.cuh"

namespace gbx {
#define GBX_PROBE(LK)                                                                                   \
    template int probe_one<LK>(const gbx_lmo&, const Layout&, int, int, const double*, const double*,  \
                               const double*, const double*, double*, double*, cudaStream_t,          \
                               std::string*);                                                          \
    template int feas_one<LK>(const gbx_lmo&, const Layout&, int, const double*, const double*,        \
                              const uint8_t*, uint8_t*, cudaStream_t, std::string*);
GBX_PROBE(GBX_LMO_BOX)
GBX_PROBE(GBX_LMO_SIMPLEX)
GBX_PROBE(GBX_LMO_EQUALITY_SIMPLEX)
GBX_PROBE(GBX_LMO_BIRKHOFF)
GBX_PROBE(GBX_LMO_CARDINALITY)
GBX_PROBE(GBX_LMO_LINKED_CARDINALITY)
#undef GBX_PROBE
}  // namespace gbx
