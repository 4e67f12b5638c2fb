// bulk_n5.cu -- step-kernel instantiations for NGLL = 5.
#include "bulk_inst.cuh"

namespace sem2d {
int launch_bulk_n5(const BulkConfig &c) { return launch_for_n<5>(c); }
int configure_bulk_n5(const BulkConfig &c) { return configure_for_n<5>(c); }
int occupancy_bulk_n5(const BulkConfig &c) { return occupancy_for_n<5>(c); }
size_t bulk_smem_n5(int ndof, int mixed, int nplanes) { return smem_for_n<5>(ndof, mixed, nplanes); }
int strip_width_n5() { return strip_width_for_n<5>(); }
int strip_batch_rows_n5() { return strip_batch_rows_for_n<5>(); }
int launch_batch_n5(const BulkConfig &c, const BatchLaunch &b) { return launch_batch_for_n<5>(c, b); }
size_t params_bytes_n5(int mixed) { return params_bytes_for_n<5>(mixed); }
void fill_params_n5(const BulkConfig &c, void *out) { fill_params_for_n<5>(c, out); }
}  // namespace sem2d
