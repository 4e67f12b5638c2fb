// bulk_n3.cu -- step-kernel instantiations for NGLL = 3.
#include "bulk_inst.cuh"

namespace sem2d {
int launch_bulk_n3(const BulkConfig &c) { return launch_for_n<3>(c); }
int configure_bulk_n3(const BulkConfig &c) { return configure_for_n<3>(c); }
int occupancy_bulk_n3(const BulkConfig &c) { return occupancy_for_n<3>(c); }
size_t bulk_smem_n3(int ndof, int mixed, int nplanes) { return smem_for_n<3>(ndof, mixed, nplanes); }
int strip_width_n3() { return strip_width_for_n<3>(); }
int strip_batch_rows_n3() { return strip_batch_rows_for_n<3>(); }
int launch_batch_n3(const BulkConfig &c, const BatchLaunch &b) { return launch_batch_for_n<3>(c, b); }
size_t params_bytes_n3(int mixed) { return params_bytes_for_n<3>(mixed); }
void fill_params_n3(const BulkConfig &c, void *out) { fill_params_for_n<3>(c, out); }
}  // namespace sem2d
