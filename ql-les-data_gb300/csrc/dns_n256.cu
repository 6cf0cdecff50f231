// Explicit instantiation of the N=256 DNS kernels and launch table.
#include "dns_ops.cuh"

namespace l3es {
template DnsTable make_dns_table<256>();
}  // namespace l3es
