// The reference's own callers compiled against the drop-in header.
//
// The reference's headers AProductCore.h and DDAModel.h are replaced by
// tdda.hpp: their include guards are defined first, so the reference's
// ObjDDAModel.h finds the drop-in classes under the reference's names.  The
// reference's ObjDDAModel.cpp (the point-field objective, ObjDDAModel.cpp:20-96)
// is compiled unchanged, where it lies in the reference checkout, as part of
// this unit; CoreStructure.cpp, Space.cpp, SpacePara.cpp, Structure.cpp,
// tools.cpp and FilterOption.cpp are compiled unchanged beside it
// (oracle/Makefile target `dropin`).  main() follows the reference's
// "DDA input" task (main.cpp:165-251): structure from a geometry and its
// densities, AProductCore, DDAModel, bicgstab, update_E_in_structure, solve_E,
// then the objective's GetVal.
//
//   dropin_reference Nx Ny Nz   (needs a CUDA device to run; the test only builds it)
#include <cstdlib>
#include <iostream>

#include "CoreStructure.h"  // the reference's structure classes (Eigen through Structure.h)
#include "Tools.h"          // build_a_bulk (tools.cpp:497-510)

#define TOPO_APRODUCTCORE_H_
#define TOPO_DDAMODEL_H_
#include "tdda.hpp"
using AProductCore = tdda::AProductCore;
using DDAModel = tdda::DDAModelT<VectorXcd>;

#include "ObjDDAModel.cpp"

int main(int argc, char** argv) {
    const int Nx = argc > 3 ? std::atoi(argv[1]) : 10, Ny = argc > 3 ? std::atoi(argv[2]) : 10,
              Nz = argc > 3 ? std::atoi(argv[3]) : 4;
    // main.cpp:165-226 with the geometry and densities given in memory
    int N = 0;
    VectorXi total_space = build_a_bulk(Nx, Ny, Nz);
    vector<Structure> ln;
    Space S(&total_space, Nx, Ny, Nz, N, &ln);
    VectorXi inputGeo = build_a_bulk(Nx, Ny, Nz);
    VectorXd inputDiel = VectorXd::Constant(Nx * Ny * Nz, 0.5);
    Structure s1(S.get_total_space(), &inputGeo);
    S = S + s1;
    Vector3i bind(1, 1, 1);
    SpacePara spacepara(&S, bind, &inputGeo, &inputDiel);
    const double d = 10.0, lam = 500.0;
    CoreStructure CStr(&spacepara, d);
    Vector3d n_K(0.0, 0.0, 1.0), n_E0(1.0, 0.0, 0.0);
    const double E0 = 1.0;
    VectorXcd material(2);
    material << std::complex<double>(1.0, 0.0), std::complex<double>(4.0, 0.1);
    const double nback = std::sqrt(std::real(material(0)));
    // main.cpp:245-251
    AProductCore Core(&CStr, lam, material, nback, "LDR");
    DDAModel TestModel(&Core, n_K, E0, n_E0);
    TestModel.bicgstab(10000, 1e-5);
    TestModel.update_E_in_structure();
    TestModel.solve_E();
    // the objective of the reference's "DDA input" loop (main.cpp:252-260)
    vector<double> objPara{d * (Nx - 1) / 2.0, d * (Ny - 1) / 2.0, d * (Nz - 1) + 100.0};
    ObjPointEDDAModel obj(objPara, &TestModel);
    obj.Reset();
    std::cout << "GetVal " << obj.GetVal() << " ITERATION " << TestModel.get_ITERATION() << std::endl;
    // the getters the reference's callers use, in the reference's types
    VectorXi* R = Core.get_R();
    VectorXd* diel_old = Core.get_diel_old();
    VectorXcd* mat = Core.get_material();
    Matrix3cd A = Core.A_dic_generator(10.0, 0.0, 0.0);
    Vector3d nE = TestModel.get_nE0();
    std::cout << (*R)(3) << " " << (*diel_old)(0) << " " << (*mat)(1) << " " << A(0, 0) << " " << nE(0) << std::endl;
    return 0;
}
