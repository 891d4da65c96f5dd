// FP64 instantiations of the lattice preconditioner's pass kernels
// (lattice_kernels.cuh), compiled apart from the FP32 ones in lattice.cu.
#include "lattice_kernels.cuh"

namespace sglat {

PassXFn<double> pass_x_fn_f64(int LGL) { return local_pass_x_fn<double>(LGL); }
PassYFn<double> pass_y_fn_f64(int LGL) { return local_pass_y_fn<double>(LGL); }
PassYFn<double> pass_yb_fn_f64(int LGL) { return local_pass_yb_fn<double>(LGL); }

}  // namespace sglat
