// tdda_pass_z.cu -- z-axis passes (K1, K5) compiled for the z FFT lengths of
// the common lattices (Nz = 10, 16, 20, 24 -> Mz = 20, 32, 40, 48), 56 and 64.
#include "tdda_passes.cuh"

namespace tdda {

bool ct_has_z(int Mz) { return Mz == 20 || Mz == 32 || Mz == 40 || Mz == 48 || Mz == 56 || Mz == 64; }

template <typename T> bool pass_ct_z(int pass, int mode, const PassArgs<T>& a, cudaError_t* err) {
    if (pass != PASS_ZFWD && pass != PASS_ZINV) return false;
    switch (a.g.pz.M) {
        case 20: *err = dev::PassLaunch<T, 20>::run_z(pass, mode, a); return true;
        case 32: *err = dev::PassLaunch<T, 32>::run_z(pass, mode, a); return true;
        case 40: *err = dev::PassLaunch<T, 40>::run_z(pass, mode, a); return true;
        case 48: *err = dev::PassLaunch<T, 48>::run_z(pass, mode, a); return true;
        case 56: *err = dev::PassLaunch<T, 56>::run_z(pass, mode, a); return true;
        case 64: *err = dev::PassLaunch<T, 64>::run_z(pass, mode, a); return true;
        default: return false;
    }
}
template bool pass_ct_z<float>(int, int, const PassArgs<float>&, cudaError_t*);
template bool pass_ct_z<double>(int, int, const PassArgs<double>&, cudaError_t*);

cudaError_t configure_pass_ct_z() {
    cudaError_t e = cudaSuccess;
    if (!e) e = dev::PassLaunch<float, 20>::configure_z();
    if (!e) e = dev::PassLaunch<float, 32>::configure_z();
    if (!e) e = dev::PassLaunch<float, 40>::configure_z();
    if (!e) e = dev::PassLaunch<float, 48>::configure_z();
    if (!e) e = dev::PassLaunch<float, 56>::configure_z();
    if (!e) e = dev::PassLaunch<float, 64>::configure_z();
    if (!e) e = dev::PassLaunch<double, 20>::configure_z();
    if (!e) e = dev::PassLaunch<double, 32>::configure_z();
    if (!e) e = dev::PassLaunch<double, 40>::configure_z();
    if (!e) e = dev::PassLaunch<double, 48>::configure_z();
    if (!e) e = dev::PassLaunch<double, 56>::configure_z();
    if (!e) e = dev::PassLaunch<double, 64>::configure_z();
    return e;
}

}  // namespace tdda
