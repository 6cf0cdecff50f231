// Explicit instantiation of the N=8 DNS kernels and launch table (coarse grids).
#include "dns_ops.cuh"

namespace l3es {
template DnsTable make_dns_table<8>();
}  // namespace l3es
