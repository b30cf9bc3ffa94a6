/*
 * shim.cpp -- CPU implementation of the cuFFT / CUDA-runtime stand-ins and a
 * host restatement of the reference's four kernel wrappers (kernel.cu:3-125:
 * A2As, B2Bs, Conv, Conv2B), so that the reference's own AProductCore.cpp /
 * DDAModel.cpp run unchanged on the CPU.  Checker infrastructure only: it is
 * linked into oracle/_ref/ref_driver and nothing else.
 */
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <set>
#include <vector>

#include "cuda_runtime_api.h"
#include "cufft.h"
#include "Kernel.h"

extern "C" {
#include "../cfft.h"
}

namespace {
std::mutex g_mu;
std::set<void*> g_live;
struct Plan { int n0, n1, n2; bool live; };
std::vector<Plan> g_plans;
}  // namespace

cudaError_t cudaMalloc(void** ptr, size_t size) {
    *ptr = std::calloc(size ? size : 1, 1);
    if (!*ptr) return 2;
    std::lock_guard<std::mutex> lk(g_mu);
    g_live.insert(*ptr);
    return 0;
}

cudaError_t cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind) {
    std::memmove(dst, src, count);
    return 0;
}

cudaError_t cudaFree(void* ptr) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_live.find(ptr);
    if (it == g_live.end()) return 0;
    g_live.erase(it);
    std::free(ptr);
    return 0;
}

cufftResult cufftPlan3d(cufftHandle* plan, int nx, int ny, int nz, cufftType) {
    if (nx < 1 || ny < 1 || nz < 1) return CUFFT_INVALID_VALUE;
    std::lock_guard<std::mutex> lk(g_mu);
    g_plans.push_back(Plan{nx, ny, nz, true});
    *plan = (cufftHandle)(g_plans.size() - 1);
    return CUFFT_SUCCESS;
}

cufftResult cufftExecZ2Z(cufftHandle plan, cufftDoubleComplex* idata, cufftDoubleComplex* odata, int direction) {
    Plan p;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (plan < 0 || plan >= (int)g_plans.size() || !g_plans[plan].live) return CUFFT_INVALID_PLAN;
        p = g_plans[plan];
    }
    size_t n = (size_t)p.n0 * p.n1 * p.n2;
    if (odata != idata) std::memmove(odata, idata, n * sizeof(cufftDoubleComplex));
#ifdef SHIM_FAST_FFT
    // timing build (oracle/_ref/ref_timer): Bluestein for the prime lengths of the 2N - 1 grid
    if (oc_fft3d_fast(p.n0, p.n1, p.n2, reinterpret_cast<oc_cplx*>(odata), direction < 0 ? -1 : 1))
        return CUFFT_ALLOC_FAILED;
#else
    if (oc_fft3d(p.n0, p.n1, p.n2, reinterpret_cast<oc_cplx*>(odata), direction < 0 ? -1 : 1)) return CUFFT_ALLOC_FAILED;
#endif
    return CUFFT_SUCCESS;
}

cufftResult cufftDestroy(cufftHandle plan) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (plan >= 0 && plan < (int)g_plans.size()) g_plans[plan].live = false;
    return CUFFT_SUCCESS;
}

/* kernel.cu:3-30 -- AoS (re, im) x {00,01,02,11,12,22} -> six arrays */
void A2As(double* A, cufftDoubleComplex* A00, cufftDoubleComplex* A01, cufftDoubleComplex* A02,
          cufftDoubleComplex* A11, cufftDoubleComplex* A12, cufftDoubleComplex* A22, int NxFFT, int NyFFT, int NzFFT) {
    cufftDoubleComplex* out[6] = {A00, A01, A02, A11, A12, A22};
    size_t n = (size_t)NxFFT * NyFFT * NzFFT;
    for (size_t g = 0; g < n; g++)
        for (int l = 0; l < 6; l++) { out[l][g].x = A[2 * l + 12 * g]; out[l][g].y = A[1 + 2 * l + 12 * g]; }
}

/* kernel.cu:44-62 -- AoS (re, im) x {x,y,z} -> three arrays */
void B2Bs(double* bDev, cufftDoubleComplex* bx, cufftDoubleComplex* by, cufftDoubleComplex* bz, int NxFFT, int NyFFT, int NzFFT) {
    cufftDoubleComplex* out[3] = {bx, by, bz};
    size_t n = (size_t)NxFFT * NyFFT * NzFFT;
    for (size_t g = 0; g < n; g++)
        for (int l = 0; l < 3; l++) { out[l][g].x = bDev[2 * l + 6 * g]; out[l][g].y = bDev[1 + 2 * l + 6 * g]; }
}

static inline cufftDoubleComplex cm(cufftDoubleComplex a, cufftDoubleComplex b) {
    cufftDoubleComplex c;
    c.x = a.x * b.x - a.y * b.y;
    c.y = a.x * b.y + a.y * b.x;
    return c;
}
static inline cufftDoubleComplex ca(cufftDoubleComplex a, cufftDoubleComplex b) {
    cufftDoubleComplex c;
    c.x = a.x + b.x;
    c.y = a.y + b.y;
    return c;
}

/* kernel.cu:74-85 -- symmetric 3x3 spectral product */
void Conv(cufftDoubleComplex* Cx, cufftDoubleComplex* Cy, cufftDoubleComplex* Cz, cufftDoubleComplex* A00,
          cufftDoubleComplex* A01, cufftDoubleComplex* A02, cufftDoubleComplex* A11, cufftDoubleComplex* A12,
          cufftDoubleComplex* A22, cufftDoubleComplex* bx, cufftDoubleComplex* by, cufftDoubleComplex* bz,
          int NxFFT, int NyFFT, int NzFFT) {
    size_t n = (size_t)NxFFT * NyFFT * NzFFT;
    for (size_t g = 0; g < n; g++) {
        Cx[g] = ca(ca(cm(A00[g], bx[g]), cm(A01[g], by[g])), cm(A02[g], bz[g]));
        Cy[g] = ca(ca(cm(A01[g], bx[g]), cm(A11[g], by[g])), cm(A12[g], bz[g]));
        Cz[g] = ca(ca(cm(A02[g], bx[g]), cm(A12[g], by[g])), cm(A22[g], bz[g]));
    }
}

/* kernel.cu:97-115 -- three arrays -> AoS (re, im) x {x,y,z} */
void Conv2B(cufftDoubleComplex* Cx, cufftDoubleComplex* Cy, cufftDoubleComplex* Cz, double* bDev, int NxFFT, int NyFFT, int NzFFT) {
    cufftDoubleComplex* in[3] = {Cx, Cy, Cz};
    size_t n = (size_t)NxFFT * NyFFT * NzFFT;
    for (size_t g = 0; g < n; g++)
        for (int l = 0; l < 3; l++) { bDev[2 * l + 6 * g] = in[l][g].x; bDev[1 + 2 * l + 6 * g] = in[l][g].y; }
}
