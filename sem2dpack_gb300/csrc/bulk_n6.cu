// bulk_n6.cu -- bulk kernel instantiations for NGLL = 6.
#include "bulk_inst.cuh"

namespace sem2d {
int launch_bulk_n6(const BulkConfig &c) { return launch_for_n<6>(c); }
int configure_bulk_n6(const BulkConfig &c) { return configure_for_n<6>(c); }
int occupancy_bulk_n6(const BulkConfig &c) { return occupancy_for_n<6>(c); }
size_t bulk_smem_n6(int ndof, int mixed, int tn, int on, int nmat, int kv, int me) {
  return smem_for_n<6>(ndof, mixed, tn, on, nmat, kv, me);
}
}  // namespace sem2d
