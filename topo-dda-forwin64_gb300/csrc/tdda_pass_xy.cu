// tdda_pass_xy.cu -- y and x passes (K2, K3, K4) compiled for the x / y FFT
// lengths of the common lattices (N = 20, 64, 80, 96 -> M = 40, 128, 160, 192).
#include "tdda_passes.cuh"

namespace tdda {

bool ct_has_xy(int M) { return M == 40 || M == 128 || M == 160 || M == 192; }
bool xpass2_length(int M) { return ct_has_xy(M) || xpass2_length2(M); }

template <typename T> bool pass_ct_xy(int pass, int mode, const PassArgs<T>& a, cudaError_t* err) {
    (void)mode;
    const bool y = pass == PASS_YFWD || pass == PASS_YINV;
    if (!y && pass != PASS_XPASS) return false;
    if constexpr (sizeof(T) == 4) {  // FP32: the register form on the two-stage plans
        if (!y && a.g.x_form == 0) {
            switch (a.g.px.M) {
#define TDDA_X2(M)                                                                       \
    case M: *err = dev::X2Launch<T, M>::run(a); return true;
                TDDA_X2(40)
                TDDA_X2(128)
                TDDA_X2(160)
                TDDA_X2(192)
#undef TDDA_X2
                default: break;
            }
        }
    }
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
    if (!e) e = dev::X2Launch<float, 40>::configure();
    if (!e) e = dev::X2Launch<float, 128>::configure();
    if (!e) e = dev::X2Launch<float, 160>::configure();
    if (!e) e = dev::X2Launch<float, 192>::configure();
    return e;
}

}  // namespace tdda
