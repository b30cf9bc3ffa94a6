// tdda_pass_dd.cu -- the A-product in double-float arithmetic (dd: FP32 pairs,
// about 44 significant bits), used for the residual r = E - (A P + al P) of the
// mixed-precision refinement.  The FP64 pass structure (z, y, x, y, z) with the
// compile-time plans of the common lengths (dd_lengths(); other grids keep the
// FP64 residual product); the
// gather reads the FP64 P and the scatter writes the FP64 r, r0, p and |r|^2,
// converting at the vectors.  GB300's FP64 pipe is narrow; these passes run on
// the FP32 pipes.
#include "tdda_passes.cuh"

namespace tdda {

namespace {

template <int CM> cudaError_t run_pass(int pass, const PassArgs<dd>& a) {
    using L = dev::PassLaunch<dd, CM>;
    if (pass == PASS_ZFWD || pass == PASS_ZINV) return L::run_z(pass, 0, a);
    if (pass == PASS_YFWD || pass == PASS_YINV) return L::run_y(pass, a);
    return L::run_x(a);
}

cudaError_t dispatch(int pass, const PassArgs<dd>& a) {
    const bool z = pass == PASS_ZFWD || pass == PASS_ZINV;
    const bool y = pass == PASS_YFWD || pass == PASS_YINV;
    const int M = z ? a.g.pz.M : (y ? a.g.py.M : a.g.px.M);
    if (z) {
        switch (M) {
            
            case 32: return run_pass<32>(pass, a);
            
            
            default: return cudaErrorInvalidValue;
        }
    }
    switch (M) {
        
        case 128: return run_pass<128>(pass, a);
        
        
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool dd_lengths(const Geom& g) { return g.pz.M == 32 && g.py.M == 128 && g.px.M == 128; }

cudaError_t launch_residual_dd(const Geom& g, int nrhs, const RhsVecs<dd>* rhs, const dd2* green, const dd2* twx,
                               const dd2* twy, const dd2* twz, const int* cellmap, dd2* grid, cudaStream_t stream) {
    const PassArgs<dd> a{g, nrhs, rhs, green, twx, twy, twz, cellmap, grid, stream, 0, 0};
    const int passes[5] = {PASS_ZFWD, PASS_YFWD, PASS_XPASS, PASS_YINV, PASS_ZINV};
    for (int k = 0; k < 5; k++) {
        const cudaError_t e = dispatch(passes[k], a);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t configure_pass_dd() {
    cudaError_t e = cudaSuccess;
    if (!e) e = dev::PassLaunch<dd, 32>::configure_z();
    if (!e) e = dev::PassLaunch<dd, 128>::configure_xy();
    return e;
}

}  // namespace tdda
