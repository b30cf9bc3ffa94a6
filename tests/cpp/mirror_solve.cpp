// Solves one lattice through the C++ drop-in (tdda.hpp) with the reference's
// call sequence (main.cpp:245-251), then evaluates the field at the lattice
// points RResult (solve_E, DDAModel.cpp:530-565), and writes ITERATION, P,
// Einternal and EResult to a file for tests/test_cpp_mirror.py to check
// against the oracle.
//
//   mirror_solve Nx Ny Nz d lam eps_re eps_im tol precision(0 FP64, 1 FP32+refine, 2 Jacobi) out.bin
// densities: rho_i = 0.5 + 0.5 sin(0.37 i), the same in the Python test.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../topo-dda-forwin64_gb300/cpp/tdda.hpp"

// the reference CoreStructure's getters, on plain vectors
struct Vec {
    std::vector<double> v;
    double operator()(size_t i) const { return v[i]; }
    size_t size() const { return v.size(); }
};
struct IVec {
    std::vector<int> v;
    int operator()(size_t i) const { return v[i]; }
    size_t size() const { return v.size(); }
};
struct Structure {
    int Nx, Ny, Nz, N;
    double d;
    IVec R;
    Vec diel_old;
    int get_N() { return N; }
    int get_Nx() { return Nx; }
    int get_Ny() { return Ny; }
    int get_Nz() { return Nz; }
    double get_d() { return d; }
    IVec* get_R() { return &R; }
    Vec* get_diel_old() { return &diel_old; }
};

int main(int argc, char** argv) {
    if (argc != 11) {
        std::fprintf(stderr, "usage: mirror_solve Nx Ny Nz d lam eps_re eps_im tol precision out.bin\n");
        return 2;
    }
    Structure S;
    S.Nx = std::atoi(argv[1]);
    S.Ny = std::atoi(argv[2]);
    S.Nz = std::atoi(argv[3]);
    S.d = std::atof(argv[4]);
    const double lam = std::atof(argv[5]);
    const std::complex<double> em(std::atof(argv[6]), std::atof(argv[7]));
    const double tol = std::atof(argv[8]);
    const int precision = std::atoi(argv[9]);
    S.N = S.Nx * S.Ny * S.Nz;
    for (int x = 0; x < S.Nx; x++)  // build_a_bulk order (tools.cpp:497-510)
        for (int y = 0; y < S.Ny; y++)
            for (int z = 0; z < S.Nz; z++) {
                S.R.v.push_back(x);
                S.R.v.push_back(y);
                S.R.v.push_back(z);
            }
    for (int i = 0; i < S.N; i++) {
        const double rho = 0.5 + 0.5 * std::sin(0.37 * i);
        for (int j = 0; j < 3; j++) S.diel_old.v.push_back(rho);
    }
    std::vector<std::complex<double>> material = {1.0, em};
    const double nK[3] = {0, 0, 1}, nE0[3] = {1, 0, 0};
    tdda::AProductCore Core(&S, lam, material, 1.0, "LDR");
    // RResult: lattice points (units of d) above, beside, past a corner of and far from the box
    const std::vector<int> RResult = {S.Nx / 2, S.Ny / 2, S.Nz + 10, -5, S.Ny / 2, S.Nz / 2,
                                      S.Nx + 3, -2, -4, 2 * S.Nx, 2 * S.Ny, 2 * S.Nz};
    tdda::DDAModel TestModel(&Core, nK, 1.0, nE0, &RResult, false);
    if (precision == 0)
        TestModel.bicgstab(100000, tol);
    else if (precision == 2)
        TestModel.bicgstab_jacobi(100000, tol);
    else
        TestModel.bicgstab_mixed(100000, tol);
    TestModel.update_E_in_structure();
    TestModel.solve_E();
    FILE* f = std::fopen(argv[10], "wb");
    if (!f) return 2;
    const int it = TestModel.get_ITERATION();
    std::fwrite(&it, 4, 1, f);
    std::fwrite(TestModel.get_P()->data(), 16, TestModel.get_P()->size(), f);
    std::fwrite(TestModel.get_Einternal()->data(), 16, TestModel.get_Einternal()->size(), f);
    std::fwrite(TestModel.get_EResult()->data(), 16, TestModel.get_EResult()->size(), f);
    TestModel.output_to_file(std::string(argv[10]) + ".", 3, 1);  // <out>.Model_results1it3.txt
    // the periodic constructor on the same structure (AProductCore.cpp:251-536): the product of
    // the solved P and one image tensor
    tdda::AProductCore PCore(&S, lam, material, 1.0, 2, 1, S.Nx * S.d, S.Ny * S.d, "LDR");
    const std::vector<std::complex<double>> y = PCore.Aproduct(*TestModel.get_P());
    std::fwrite(y.data(), 16, y.size(), f);
    const auto A = PCore.A_dic_generator(10.0, 20.0, 5.0, 1, -1);
    for (int i = 0; i < 3; i++) std::fwrite(A[i].data(), 16, 3, f);
    std::fclose(f);
    std::printf("ITERATION %d P[0] %.17g %.17g\n", it, (*TestModel.get_P())[0].real(), (*TestModel.get_P())[0].imag());
    return 0;
}
