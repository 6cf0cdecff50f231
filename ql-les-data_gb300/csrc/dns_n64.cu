// Explicit instantiation of the N=64 DNS kernels and launch table.
#include "dns_ops.cuh"

namespace l3es {
template DnsTable make_dns_table<64>();
}  // namespace l3es
