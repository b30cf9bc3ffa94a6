// tdda_pass_dd_192.cu -- double-float A-product passes for x/y length 192 and z length 48
// (the dispatch and the rest are in tdda_pass_dd.cu; one unit per length pair
// keeps the build parallel).
#include "tdda_passes.cuh"

namespace tdda {

cudaError_t dd_pass_z48(int pass, const PassArgs<dd>& a) { return dev::PassLaunch<dd, 48>::run_z(pass, 0, a); }
cudaError_t dd_pass_xy192(int pass, const PassArgs<dd>& a) {
    using L = dev::PassLaunch<dd, 192>;
    return (pass == PASS_YFWD || pass == PASS_YINV) ? L::run_y(pass, a) : L::run_x(a);
}
cudaError_t configure_dd_192_48() {
    cudaError_t e = dev::PassLaunch<dd, 48>::configure_z();
    return e != cudaSuccess ? e : dev::PassLaunch<dd, 192>::configure_xy();
}

}  // namespace tdda
