/*
 * tdda_oracle.h -- CPU restatement of the reference's DDA solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA
 * product path: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  It is never linked into libtdda.
 *
 * It restates, in plain C, what the reference computes on this path:
 *   AProductCore ctor (Green tensor + spectra)  AProductCore.cpp:12-249
 *   AProductCore::LDR_inter                     AProductCore.cpp:588-623
 *   AProductCore::Aproduct                      AProductCore.cpp:697-758
 *   DDAModel ctor (E_inc, diel, al)             DDAModel.cpp:12-69
 *   DDAModel::bicgstab                          DDAModel.cpp:131-260
 *   DDAModel::UpdateAlpha / Aproductwithalb     DDAModel.cpp:470-487, 577-586
 *   DDAModel::update_E_in_structure             DDAModel.cpp:567-575
 *   Get_Alpha (LDR polarisability)              tools.cpp:617-630
 * Parity pin: tests/golden/ holds outputs of the reference's own sources
 * (compiled here with a CPU stand-in for cuFFT, oracle/Makefile target
 * `ref`), and tests/test_oracle_golden.py checks this restatement against
 * them.
 *
 * Complex vectors are interleaved doubles (re, im), i.e. the storage of
 * std::complex<double> / Eigen::VectorXcd.  Dipole vectors are AoS
 * [Px, Py, Pz] per dipole, dipole order = order of R.
 */
#ifndef ORACLE_TDDA_ORACLE_H_
#define ORACLE_TDDA_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* status codes of or_model_bicgstab */
#define OR_CONVERGED 0
#define OR_BREAKDOWN 1
#define OR_MAXITER 2

void or_normalize_material(int nmat, const double* mat_in, double nback, double* mat_out);
void or_ldr_inter(double K, double x, double y, double z, double* out12);
/* Si(x), Ci(x) for x > 0 (A&S 5.2.14, 5.2.16, 5.2.23, 5.1.22) */
void or_sici(double x, double* si, double* ci);
/* FCD tensor (AProductCore.cpp:625-695) with the interpolated Si/Ci tables */
void or_fcd_inter(double K, double d, double x, double y, double z, double* out12);
void or_get_alpha(double lam, double K, double d, double eps_re, double eps_im,
                  const double* nE0, const double* nK, double* out2);

typedef struct or_core or_core;

/* Mx/My/Mz <= 0 selects the reference's grid 2N-1 per axis; any value
 * >= 2N-1 gives the same linear convolution. */
or_core* or_core_create(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam,
                        double nback, int nmat, const double* material, int Mx, int My, int Mz);
/* the periodic constructor (AProductCore.cpp:251-536): the tensor at each
 * offset is the sum of its images over m in [-MAXm, MAXm], n in [-MAXn, MAXn]
 * with periods Lm (x) and Ln (y), each damped by exp(-(0.01 K r)^4) */
or_core* or_core_create_periodic(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam, double nback,
                                 int nmat, const double* material, int MAXm, int MAXn, double Lm, double Ln,
                                 int Mx, int My, int Mz);
/* general constructor: method 0 LDR, 1 FCD; periodic as or_core_create_periodic */
or_core* or_core_create_method(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam, double nback,
                               int nmat, const double* material, int method, int periodic, int MAXm, int MAXn,
                               double Lm, double Ln, int Mx, int My, int Mz);
void or_core_destroy(or_core* c);
void or_core_set_pruned(or_core* c, int pruned);
double or_core_K(const or_core* c);
void or_core_material(const or_core* c, double* out);
void or_core_grid(const or_core* c, int* out3);
/* y = A_offdiag b (3N complex) */
int or_aproduct(or_core* c, const double* b, double* y);
/* the same product by the O(N^2) direct sum of LDR tensors */
int or_aproduct_direct(int N, const int* R, double d, double K, const double* b, double* y);

typedef struct or_model or_model;
or_model* or_model_create(or_core* c, const double* nK, double E0, const double* nE0,
                          const double* diel_old);
void or_model_destroy(or_model* m);
int or_model_update_alpha(or_model* m, const double* diel_old);
void or_model_change_E(or_model* m, const double* E);
void or_model_reset_E(or_model* m);
void or_model_initialize_P(or_model* m, const double* P);
int or_model_aproduct_with_alb(or_model* m, const double* b, double* y);
int or_model_bicgstab(or_model* m, int max_it, double max_err, int* iterations, double* error);
void or_model_update_E_in_structure(or_model* m);
/* E(r) = E_ext(r) - sum_i A(r - d R_i) P_i at npts points (nm) into
 * E_out (npts x 3 complex) */
void or_model_field_at(const or_model* m, int npts, const double* pts, double* E_out);
/* what: 0 P, 1 E, 2 al, 3 diel, 4 Einternal (each 3N complex) */
void or_model_get(const or_model* m, int what, double* out);

#ifdef __cplusplus
}
#endif

#endif
