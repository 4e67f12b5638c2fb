// bulk_n5.cu -- bulk kernel instantiations for NGLL = 5.
#include "bulk_inst.cuh"

namespace sem2d {
int launch_bulk_n5(const BulkConfig &c) { return launch_for_n<5>(c); }
int configure_bulk_n5(const BulkConfig &c) { return configure_for_n<5>(c); }
int occupancy_bulk_n5(const BulkConfig &c) { return occupancy_for_n<5>(c); }
size_t bulk_smem_n5(int ndof, int mixed, int tn, int on, int nmat, int kv, int me) {
  return smem_for_n<5>(ndof, mixed, tn, on, nmat, kv, me);
}
}  // namespace sem2d
