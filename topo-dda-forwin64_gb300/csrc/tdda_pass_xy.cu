// tdda_pass_xy.cu -- y and x passes (K2, K3, K4) compiled for the x / y FFT
// lengths of the common lattices (N = 20, 64, 80, 96 -> M = 40, 128, 160, 192).
#include "tdda_passes.cuh"

namespace tdda {

bool ct_has_xy(int M) { return M == 40 || M == 128 || M == 160 || M == 192; }

template <typename T> bool pass_ct_xy(int pass, int mode, const PassArgs<T>& a, cudaError_t* err) {
    (void)mode;
    const bool y = pass == PASS_YFWD || pass == PASS_YINV;
    if (!y && pass != PASS_XPASS) return false;
    switch (y ? a.g.py.M : a.g.px.M) {
#define TDDA_XY(M)                                                                                      \
    case M:                                                                                             \
        *err = y ? dev::PassLaunch<T, M>::run_y(pass, a) : dev::PassLaunch<T, M>::run_x(a);              \
        return true;
        TDDA_XY(40)
        TDDA_XY(128)
        TDDA_XY(160)
        TDDA_XY(192)
#undef TDDA_XY
        default: return false;
    }
}
template bool pass_ct_xy<float>(int, int, const PassArgs<float>&, cudaError_t*);
template bool pass_ct_xy<double>(int, int, const PassArgs<double>&, cudaError_t*);

cudaError_t configure_pass_ct_xy() {
    cudaError_t e = cudaSuccess;
    if (!e) e = dev::PassLaunch<float, 40>::configure_xy();
    if (!e) e = dev::PassLaunch<float, 128>::configure_xy();
    if (!e) e = dev::PassLaunch<float, 160>::configure_xy();
    if (!e) e = dev::PassLaunch<float, 192>::configure_xy();
    if (!e) e = dev::PassLaunch<double, 40>::configure_xy();
    if (!e) e = dev::PassLaunch<double, 128>::configure_xy();
    if (!e) e = dev::PassLaunch<double, 160>::configure_xy();
    if (!e) e = dev::PassLaunch<double, 192>::configure_xy();
    return e;
}

}  // namespace tdda
