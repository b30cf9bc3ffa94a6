// tdda_pass_zy.cu -- fused z+y passes (k_zyfwd, k_yzinv) of the FP32
// A-product, compiled for the (My, Mz) planes of the common lattices
// (Ny x Nz = 20x10, 64x16, 80x20, 96x24 -> 40x20, 128x32, 160x40, 192x48).
#include "tdda_passes.cuh"

namespace tdda {

bool zy_fused(const Geom& g, bool fp32) {
    if (!fp32) return false;
    const int My = g.py.M, Mz = g.pz.M;
    return (My == 40 && Mz == 20) || (My == 128 && Mz == 32) || (My == 160 && Mz == 40) || (My == 192 && Mz == 48);
}

template <> bool pass_zy<double>(int, int, const PassArgs<double>&, cudaError_t*) { return false; }

template <> bool pass_zy<float>(int pass, int mode, const PassArgs<float>& a, cudaError_t* err) {
    if (pass != PASS_ZFWD && pass != PASS_ZINV) return false;
    const int My = a.g.py.M, Mz = a.g.pz.M;
#define TDDA_ZY(MY, MZ)                                                         \
    if (My == MY && Mz == MZ) {                                                 \
        *err = dev::ZyLaunch<float, MY, MZ>::run(pass, mode, a);                \
        return true;                                                            \
    }
    TDDA_ZY(40, 20)
    TDDA_ZY(128, 32)
    TDDA_ZY(160, 40)
    TDDA_ZY(192, 48)
#undef TDDA_ZY
    return false;
}

cudaError_t configure_pass_zy() {
    cudaError_t e = cudaSuccess;
    if (!e) e = dev::ZyLaunch<float, 40, 20>::configure();
    if (!e) e = dev::ZyLaunch<float, 128, 32>::configure();
    if (!e) e = dev::ZyLaunch<float, 160, 40>::configure();
    if (!e) e = dev::ZyLaunch<float, 192, 48>::configure();
    return e;
}

}  // namespace tdda
