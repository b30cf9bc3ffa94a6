// tdda_pass_dd_128.cu -- double-float A-product passes for x/y length 128 and z length 32
// (the dispatch and the rest are in tdda_pass_dd.cu; one unit per length pair
// keeps the build parallel).
#include "tdda_passes.cuh"

namespace tdda {

cudaError_t dd_pass_z32(int pass, const PassArgs<dd>& a) { return dev::PassLaunch<dd, 32>::run_z(pass, 0, a); }
cudaError_t dd_pass_xy128(int pass, const PassArgs<dd>& a) {
    using L = dev::PassLaunch<dd, 128>;
    return (pass == PASS_YFWD || pass == PASS_YINV) ? L::run_y(pass, a) : L::run_x(a);
}
cudaError_t configure_dd_128_32() {
    cudaError_t e = dev::PassLaunch<dd, 32>::configure_z();
    return e != cudaSuccess ? e : dev::PassLaunch<dd, 128>::configure_xy();
}

}  // namespace tdda
