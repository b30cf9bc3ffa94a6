// tdda_pass_generic.cu -- A-product pass kernels with the FFT plan read at run
// time: every 7-smooth length is served here.
#include "tdda_passes.cuh"

namespace tdda {

template <typename T> cudaError_t pass_generic(int pass, int mode, const PassArgs<T>& a) {
    return dev::PassLaunch<T, 0>::run(pass, mode, a);
}
template cudaError_t pass_generic<float>(int, int, const PassArgs<float>&);
template cudaError_t pass_generic<double>(int, int, const PassArgs<double>&);

cudaError_t configure_pass_generic() {
    cudaError_t e = dev::PassLaunch<float, 0>::configure_z();
    if (e == cudaSuccess) e = dev::PassLaunch<float, 0>::configure_xy();
    if (e == cudaSuccess) e = dev::PassLaunch<double, 0>::configure_z();
    if (e == cudaSuccess) e = dev::PassLaunch<double, 0>::configure_xy();
    return e;
}

}  // namespace tdda
