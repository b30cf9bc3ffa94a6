// tdda_pass_xy2.cu -- y and x passes compiled for the further x / y FFT lengths
// a core rounds its axes up to (32, 48, 56, 64, 80, 96, 112, 224, 256; the
// lattices of a served request stream), beside tdda_pass_xy.cu's lengths of
// the common lattices.  FP32 x passes take the register form on the two-stage
// plans (not 224 and 256, which have none that fits the registers).
#include "tdda_passes.cuh"

namespace tdda {

bool ct_has_xy2(int M) {
    return M == 32 || M == 48 || M == 56 || M == 64 || M == 80 || M == 96 || M == 112 || M == 224 || M == 256;
}
bool xpass2_length2(int M) { return M == 32 || M == 48 || M == 56 || M == 64 || M == 80 || M == 96 || M == 112; }

template <typename T> bool pass_ct_xy2(int pass, int mode, const PassArgs<T>& a, cudaError_t* err) {
    (void)mode;
    const bool y = pass == PASS_YFWD || pass == PASS_YINV;
    if (!y && pass != PASS_XPASS) return false;
    if constexpr (sizeof(T) == 4) {
        if (!y && a.g.x_form == 0) {
            switch (a.g.px.M) {
#define TDDA_X2(M)                                                         \
    case M: *err = dev::X2Launch<T, M>::run(a); return true;
                TDDA_X2(32)
                TDDA_X2(48)
                TDDA_X2(56)
                TDDA_X2(64)
                TDDA_X2(80)
                TDDA_X2(96)
                TDDA_X2(112)
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
        TDDA_XY(32)
        TDDA_XY(48)
        TDDA_XY(56)
        TDDA_XY(64)
        TDDA_XY(80)
        TDDA_XY(96)
        TDDA_XY(112)
        TDDA_XY(224)
        TDDA_XY(256)
#undef TDDA_XY
        default: return false;
    }
}
template bool pass_ct_xy2<float>(int, int, const PassArgs<float>&, cudaError_t*);
template bool pass_ct_xy2<double>(int, int, const PassArgs<double>&, cudaError_t*);

cudaError_t configure_pass_ct_xy2() {
    cudaError_t e = cudaSuccess;
#define TDDA_CFG(M)                                                                   \
    if (!e) e = dev::PassLaunch<float, M>::configure_xy();                            \
    if (!e) e = dev::PassLaunch<double, M>::configure_xy();
    TDDA_CFG(32)
    TDDA_CFG(48)
    TDDA_CFG(56)
    TDDA_CFG(64)
    TDDA_CFG(80)
    TDDA_CFG(96)
    TDDA_CFG(112)
    TDDA_CFG(224)
    TDDA_CFG(256)
#undef TDDA_CFG
    if (!e) e = dev::X2Launch<float, 32>::configure();
    if (!e) e = dev::X2Launch<float, 48>::configure();
    if (!e) e = dev::X2Launch<float, 64>::configure();
    if (!e) e = dev::X2Launch<float, 80>::configure();
    if (!e) e = dev::X2Launch<float, 96>::configure();
    if (!e) e = dev::X2Launch<float, 56>::configure();
    if (!e) e = dev::X2Launch<float, 112>::configure();
    return e;
}

}  // namespace tdda
