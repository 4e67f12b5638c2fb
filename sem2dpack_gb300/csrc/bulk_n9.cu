// bulk_n9.cu -- bulk kernel instantiations for NGLL = 9.
#include "bulk_inst.cuh"

namespace sem2d {
int launch_bulk_n9(const BulkConfig &c) { return launch_for_n<9>(c); }
int configure_bulk_n9(const BulkConfig &c) { return configure_for_n<9>(c); }
int occupancy_bulk_n9(const BulkConfig &c) { return occupancy_for_n<9>(c); }
size_t bulk_smem_n9(int ndof, int mixed, int tn, int on, int nmat, int kv, int me) {
  return smem_for_n<9>(ndof, mixed, tn, on, nmat, kv, me);
}
}  // namespace sem2d
