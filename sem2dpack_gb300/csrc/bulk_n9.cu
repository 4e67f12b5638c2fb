// bulk_n9.cu -- step-kernel instantiations for NGLL = 9.
#include "bulk_inst.cuh"

namespace sem2d {
int launch_bulk_n9(const BulkConfig &c) { return launch_for_n<9>(c); }
int configure_bulk_n9(const BulkConfig &c) { return configure_for_n<9>(c); }
int occupancy_bulk_n9(const BulkConfig &c) { return occupancy_for_n<9>(c); }
size_t bulk_smem_n9(int ndof, int mixed, int nplanes) { return smem_for_n<9>(ndof, mixed, nplanes); }
int strip_width_n9() { return strip_width_for_n<9>(); }
int strip_batch_rows_n9() { return strip_batch_rows_for_n<9>(); }
int launch_batch_n9(const BulkConfig &c, const BatchLaunch &b) { return launch_batch_for_n<9>(c, b); }
size_t params_bytes_n9(int mixed) { return params_bytes_for_n<9>(mixed); }
void fill_params_n9(const BulkConfig &c, void *out) { fill_params_for_n<9>(c, out); }
}  // namespace sem2d
