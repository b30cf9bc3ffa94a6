// tdda_pass_dd.cu -- the A-product in double-float arithmetic (dd: FP32 pairs,
// about 44 significant bits), used for the residual r = E - (A P + al P) of the
// mixed-precision refinement.  The FP64 pass structure (z, y, x, y, z) on the
// compile-time plans of the common lengths (tdda_pass_dd_<M>.cu; other grids
// keep the FP64 residual product).  The gather reads the FP64 P and the scatter
// writes the FP64 r, r0, p and |r|^2, converting at the vectors.  GB300's FP64
// pipe is narrow; these passes run on the FP32 pipes.
#include "tdda_passes.cuh"

namespace tdda {

cudaError_t dd_pass_z32(int pass, const PassArgs<dd>& a);
cudaError_t dd_pass_z48(int pass, const PassArgs<dd>& a);
cudaError_t dd_pass_z40(int pass, const PassArgs<dd>& a);
cudaError_t dd_pass_z20(int pass, const PassArgs<dd>& a);
cudaError_t dd_pass_xy128(int pass, const PassArgs<dd>& a);
cudaError_t dd_pass_xy192(int pass, const PassArgs<dd>& a);
cudaError_t dd_pass_xy160(int pass, const PassArgs<dd>& a);
cudaError_t dd_pass_xy40(int pass, const PassArgs<dd>& a);
cudaError_t configure_dd_128_32();
cudaError_t configure_dd_192_48();
cudaError_t configure_dd_160_40();
cudaError_t configure_dd_40_20();

namespace {

using PassFn = cudaError_t (*)(int, const PassArgs<dd>&);

PassFn z_pass(int M) {
    switch (M) {
        case 20: return dd_pass_z20;
        case 32: return dd_pass_z32;
        case 40: return dd_pass_z40;
        case 48: return dd_pass_z48;
        default: return nullptr;
    }
}
PassFn xy_pass(int M) {
    switch (M) {
        case 40: return dd_pass_xy40;
        case 128: return dd_pass_xy128;
        case 160: return dd_pass_xy160;
        case 192: return dd_pass_xy192;
        default: return nullptr;
    }
}

}  // namespace

bool dd_lengths(const Geom& g) { return z_pass(g.pz.M) && xy_pass(g.py.M) && xy_pass(g.px.M); }

cudaError_t launch_residual_dd(const Geom& g, int nrhs, const RhsVecs<dd>* rhs, const dd2* green, const dd2* twx,
                               const dd2* twy, const dd2* twz, const int* cellmap, dd2* grid, cudaStream_t stream) {
    if (!dd_lengths(g)) return cudaErrorInvalidValue;
    const PassArgs<dd> a{g, nrhs, rhs, green, twx, twy, twz, cellmap, grid, stream, 0, 0};
    const PassFn fz = z_pass(g.pz.M), fy = xy_pass(g.py.M), fx = xy_pass(g.px.M);
    const PassFn fns[5] = {fz, fy, fx, fy, fz};
    const int passes[5] = {PASS_ZFWD, PASS_YFWD, PASS_XPASS, PASS_YINV, PASS_ZINV};
    for (int k = 0; k < 5; k++) {
        const cudaError_t e = fns[k](passes[k], a);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t configure_pass_dd() {
    cudaError_t e = configure_dd_128_32();
    if (!e) e = configure_dd_192_48();
    if (!e) e = configure_dd_160_40();
    if (!e) e = configure_dd_40_20();
    return e;
}

}  // namespace tdda
