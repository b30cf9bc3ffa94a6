// tdda_pass_dd_160.cu -- double-float A-product passes for x/y length 160 and z length 40
// (the dispatch and the rest are in tdda_pass_dd.cu; one unit per length pair
// keeps the build parallel).
#include "tdda_passes.cuh"

namespace tdda {

cudaError_t dd_pass_z40(int pass, const PassArgs<dd>& a) { return dev::PassLaunch<dd, 40>::run_z(pass, 0, a); }
cudaError_t dd_pass_xy160(int pass, const PassArgs<dd>& a) {
    using L = dev::PassLaunch<dd, 160>;
    return (pass == PASS_YFWD || pass == PASS_YINV) ? L::run_y(pass, a) : L::run_x(a);
}
cudaError_t configure_dd_160_40() {
    cudaError_t e = dev::PassLaunch<dd, 40>::configure_z();
    return e != cudaSuccess ? e : dev::PassLaunch<dd, 160>::configure_xy();
}

}  // namespace tdda
