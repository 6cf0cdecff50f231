// Explicit instantiation of the N=16 DNS kernels and launch table.
#include "dns_ops.cuh"

namespace l3es {
template DnsTable make_dns_table<16>();
}  // namespace l3es
