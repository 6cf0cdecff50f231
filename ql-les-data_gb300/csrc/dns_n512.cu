// Explicit instantiation of the N=512 DNS kernels and launch table.
#include "dns_ops.cuh"

namespace l3es {
template DnsTable make_dns_table<512>();
}  // namespace l3es
