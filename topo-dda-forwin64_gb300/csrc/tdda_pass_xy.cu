// tdda_pass_xy.cu -- y and x passes (K2, K3, K4) compiled for the x / y FFT
// lengths of the common lattices (N = 20, 64, 80, 96 -> M = 40, 128, 160, 192).
#include "tdda_passes.cuh"

namespace tdda {

bool ct_has_xy(int M) { return M == 40 || M == 128 || M == 160 || M == 192; }
bool xpass2_length(int M) { return ct_has_xy(M) || xpass2_length2(M); }

// z-columns per block of the register-form x pass (k_xpass2), per length
template <int M> constexpr int xpass2_tile() { return M == 128 ? 16 : 8; }
// blocks per SM the register form is compiled for: 16 warps per SM (a
// register cap of 128 per thread), 24 for M = 128, whose spectra fit in 85
template <int M> constexpr int xpass2_minb() {
    return (M == 128 || M == 192 ? 24 : 16) * 32 / (xpass2_tile<M>() * x2_radix(M, 0));
}

template <typename T> bool pass_ct_xy(int pass, int mode, const PassArgs<T>& a, cudaError_t* err) {
    (void)mode;
    const bool y = pass == PASS_YFWD || pass == PASS_YINV;
    if (!y && pass != PASS_XPASS) return false;
    if constexpr (sizeof(T) == 4) {  // FP32: the register form on the two-stage plans
        if (!y) {
            switch (a.g.px.M) {
#define TDDA_X2(M)                                                                       \
    case M: *err = dev::XLaunch2<T, M, xpass2_tile<M>(), xpass2_minb<M>()>::run(a); return true;
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
    if (!e) e = dev::XLaunch2<float, 40, xpass2_tile<40>(), xpass2_minb<40>()>::configure();
    if (!e) e = dev::XLaunch2<float, 128, xpass2_tile<128>(), xpass2_minb<128>()>::configure();
    if (!e) e = dev::XLaunch2<float, 160, xpass2_tile<160>(), xpass2_minb<160>()>::configure();
    if (!e) e = dev::XLaunch2<float, 192, xpass2_tile<192>(), xpass2_minb<192>()>::configure();
    return e;
}

}  // namespace tdda
