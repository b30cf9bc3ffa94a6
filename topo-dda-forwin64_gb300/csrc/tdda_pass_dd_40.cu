// tdda_pass_dd_40.cu -- double-float A-product passes for x/y length 40 and z length 20
// (the dispatch and the rest are in tdda_pass_dd.cu; one unit per length pair
// keeps the build parallel).
#include "tdda_passes.cuh"

namespace tdda {

cudaError_t dd_pass_z20(int pass, const PassArgs<dd>& a) { return dev::PassLaunch<dd, 20>::run_z(pass, 0, a); }
cudaError_t dd_pass_xy40(int pass, const PassArgs<dd>& a) {
    using L = dev::PassLaunch<dd, 40>;
    return (pass == PASS_YFWD || pass == PASS_YINV) ? L::run_y(pass, a) : L::run_x(a);
}
cudaError_t configure_dd_40_20() {
    cudaError_t e = dev::PassLaunch<dd, 20>::configure_z();
    return e != cudaSuccess ? e : dev::PassLaunch<dd, 40>::configure_xy();
}

}  // namespace tdda
