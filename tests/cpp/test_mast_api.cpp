// Tests of the C++ mirror of MAST's API (mast_api.hpp), written the way MAST's
// own tests are (tests/material/mast_isotropic_material.cpp,
// tests/element/structural/...): build the property cards, disciplines and
// boundary conditions, assemble or solve, compare with the truth.  The truth
// here is the FP64 oracle (oracle/mast_oracle.h), itself pinned to the
// reference's known answers by tests/test_oracle_pins.py.
#include <cmath>
#include <memory>
#include <random>
#include <vector>

#include "mast_api.hpp"
#include "mast_oracle.h"
#include "mini_catch.hpp"

using MAST::Real;

static bool have_gpu() {
    char name[64];
    int sm = 0, ma = 0, mi = 0;
    return mg_device_info(name, 64, &sm, &ma, &mi) == MG_OK;
}

TEST_CASE("constant_isotropic_structural_material_3d", "[cpu],[isotropic],[material],[3D]") {
    MAST::Parameter E("E_param", 72.0e9), nu("nu_param", 0.33);
    MAST::ConstantFieldFunction E_f("E", E), nu_f("nu", nu);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(E_f);
    material.add(nu_f);
    REQUIRE(material.contains("E"));
    REQUIRE(material.contains("nu"));
    const MAST::FieldFunction<MAST::RealMatrixX> &mat_stiff = material.stiffness_matrix(3);
    MAST::RealMatrixX D;
    mat_stiff(MAST::Point(2.3, 3.1, 5.2), 2.34, D);
    double truth[36];
    or_iso_stiffness_3d(72.0e9, 0.33, truth);
    REQUIRE(D.rows() == 6 && D.cols() == 6);
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) {
            CHECK(D(i, j) == Approx(truth[6 * i + j]).margin(1e-6));
            CHECK(D(i, j) == Approx(D(j, i)));
        }
    // dC/dE with nu held: C(E = 1)
    MAST::RealMatrixX dD;
    mat_stiff.derivative(E, MAST::Point(), 0.0, dD);
    or_iso_stiffness_3d(1.0, 0.33, truth);
    for (int i = 0; i < 36; i++) CHECK(dD.data()[i] == Approx(truth[i]));
}

TEST_CASE("constant_isotropic_structural_material_2d", "[cpu],[isotropic],[material],[2D]") {
    MAST::Parameter E("E_param", 72.0e9), nu("nu_param", 0.33);
    MAST::ConstantFieldFunction E_f("E", E), nu_f("nu", nu);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(E_f);
    material.add(nu_f);
    for (int strain = 0; strain < 2; strain++) {
        MAST::RealMatrixX D;
        material.stiffness_matrix(2, strain == 1)(MAST::Point(), 0.0, D);
        double truth[9];
        or_iso_stiffness_2d(72.0e9, 0.33, strain == 0, truth);
        for (int i = 0; i < 9; i++) CHECK(D.data()[i] == Approx(truth[i]).margin(1e-6));
    }
}

TEST_CASE("constant_isotropic_thermal_conductance", "[cpu],[isotropic],[material],[thermal]") {
    MAST::Parameter k("k_param", 237.0);
    MAST::ConstantFieldFunction k_f("k_th", k);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(k_f);
    for (int dim = 1; dim <= 3; dim++) {
        MAST::RealMatrixX K;
        material.conductance_matrix(dim)(MAST::Point(), 0.0, K);
        for (int i = 0; i < dim; i++)
            for (int j = 0; j < dim; j++) CHECK(K(i, j) == Approx(i == j ? 237.0 : 0.0));
    }
}

TEST_CASE("build_cube_numbering_and_boundary_ids", "[cpu],[mesh]") {
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_cube(mesh, 4, 3, 2, 0, 4, 0, 3, 0, 2);
    std::vector<double> c(5 * 4 * 3 * 3);
    std::vector<int32_t> e(4 * 3 * 2 * 8);
    or_grid_hex8(4, 3, 2, 4, 3, 2, c.data(), e.data());
    REQUIRE(mesh.coords.size() == c.size() && mesh.conn.size() == e.size());
    for (size_t i = 0; i < c.size(); i++) CHECK(mesh.coords[i] == Approx(c[i]));
    for (size_t i = 0; i < e.size(); i++) CHECK(mesh.conn[i] == e[i]);
    CHECK(mesh.boundary_nodes(4).size() == 4 * 3);  // x = 0 face
    CHECK(mesh.boundary_nodes(2).size() == 4 * 3);  // x = max face
    CHECK(mesh.boundary_nodes(0).size() == 5 * 4);  // z = 0 face
    MAST::Mesh sq;
    MAST::MeshTools::Generation::build_square(sq, 5, 4, 0, 1, 0, 1);
    CHECK(sq.boundary_sides(1).size() == 4);  // x = 1 edge
    CHECK(sq.boundary_nodes(3).size() == 5);  // x = 0 edge
}

// MAST::NastranIO: a 3 x 2 x 2 cube written as GRID / CHEXA / SPC1 cards reads
// back as build_cube's mesh, the SPC nodes as boundary 1, the Nastran ids mapped
TEST_CASE("nastran_io_reads_a_cube", "[cpu],[mesh],[nastran]") {
    MAST::Mesh cube;
    MAST::MeshTools::Generation::build_cube(cube, 3, 2, 2, 0, 3, 0, 2, 0, 2);
    std::string deck = "$ cube\nBEGIN BULK\n";
    char line[128];
    for (int64_t n = 0; n < cube.n_nodes(); n++) {
        snprintf(line, sizeof(line), "GRID,%lld,,%g,%g,%g\n", (long long)(501 + n), cube.coords[3 * n],
                 cube.coords[3 * n + 1], cube.coords[3 * n + 2]);
        deck += line;
    }
    for (int64_t e = 0; e < cube.n_elem(); e++) {
        const int32_t *c = &cube.conn[8 * e];
        snprintf(line, sizeof(line), "CHEXA,%lld,7,%d,%d,%d,%d,%d,%d\n,%d,%d\n", (long long)(e + 1), 501 + c[0],
                 501 + c[1], 501 + c[2], 501 + c[3], 501 + c[4], 501 + c[5], 501 + c[6], 501 + c[7]);
        deck += line;
    }
    const std::vector<int64_t> clamp = cube.boundary_nodes(4);  // x = 0 face
    for (int64_t n : clamp) {
        snprintf(line, sizeof(line), "SPC1,1,123,%lld\n", (long long)(501 + n));
        deck += line;
    }
    deck += "ENDDATA\n";
    const std::string path = "nastran_io_cube.bdf";
    FILE *fp = fopen(path.c_str(), "w");
    REQUIRE(fp != nullptr);
    fputs(deck.c_str(), fp);
    fclose(fp);
    MAST::Mesh mesh;
    MAST::NastranIO io(mesh);
    io.read(path);
    REQUIRE(mesh.type == MAST::HEX8);
    REQUIRE(mesh.coords.size() == cube.coords.size() && mesh.conn.size() == cube.conn.size());
    for (size_t i = 0; i < cube.coords.size(); i++) CHECK(mesh.coords[i] == Approx(cube.coords[i]));
    for (size_t i = 0; i < cube.conn.size(); i++) CHECK(mesh.conn[i] == cube.conn[i]);
    CHECK(mesh.boundary_nodes(1) == clamp);
    CHECK(io.get_nastran_to_libmesh_node_map().at(501 + 7) == 7);
    CHECK(io.get_nastran_to_libmesh_elem_map().at(5) == 4);
    REQUIRE_THROWS(io.read("no_such_deck.bdf"));
    remove(path.c_str());
}

TEST_CASE("misuse_is_reported", "[cpu],[errors]") {
    REQUIRE_THROWS(MAST::PointLoadCondition(MAST::DIRICHLET));
    MAST::NonlinearImplicitAssembly assembly;
    REQUIRE_THROWS(assembly.problem());  // no discipline and system
    MAST::IsotropicMaterialPropertyCard material;
    REQUIRE_THROWS(material.value("E"));
    if (!have_gpu()) {
        // a complete set-up on a host without a GPU: the library's status surfaces
        MAST::Mesh mesh;
        MAST::MeshTools::Generation::build_cube(mesh, 2, 1, 1, 0, 2, 0, 1, 0, 1);
        MAST::Parameter E("E_param", 1.0), nu("nu_param", 0.3);
        MAST::ConstantFieldFunction E_f("E", E), nu_f("nu", nu);
        material.add(E_f);
        material.add(nu_f);
        MAST::Solid3DSectionElementPropertyCard section;
        section.set_material(material);
        MAST::StructuralDiscipline discipline;
        discipline.set_property_for_subdomain(0, section);
        MAST::NonlinearSystem sys;
        MAST::StructuralSystemInitialization init(sys, mesh);
        MAST::StructuralNonlinearAssemblyElemOperations ops;
        assembly.set_discipline_and_system(discipline, init, ops);
        bool ecuda = false;
        try {
            assembly.problem();
        } catch (const MAST::Error &e) {
            ecuda = (e.status == MG_ECUDA || e.status == MG_ENOMEM);
        }
        REQUIRE(ecuda);
    }
}

// config 0, written as a MAST driver: clamp x = 0, -z unit load over the x = max,
// z = 0 edge, SIMP densities, Jacobi-PCG to 1e-10, compliance and dC/drho by adjoint
TEST_CASE("hex8_simp_cantilever", "[gpu],[structural],[3D]") {
    const int nx = 24, ny = 12, nz = 12;
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_cube(mesh, nx, ny, nz, 0, nx, 0, ny, 0, nz);
    MAST::Parameter E("E_param", 1.0), nu("nu_param", 0.3);
    MAST::ConstantFieldFunction E_f("E", E), nu_f("nu", nu);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(E_f);
    material.add(nu_f);
    MAST::Solid3DSectionElementPropertyCard section;
    section.set_material(material);
    MAST::StructuralDiscipline discipline;
    discipline.set_property_for_subdomain(0, section);
    MAST::DirichletBoundaryCondition clamp;
    clamp.init(4, {0, 1, 2});
    discipline.add_dirichlet_bc(4, clamp);
    MAST::PointLoadCondition load(MAST::POINT_LOAD);
    int n_load = 0;
    for (int64_t n : mesh.boundary_nodes(2))
        if (mesh.point(n).z == 0.0) {
            load.add_node(n);
            n_load++;
        }
    load.set_load({0.0, 0.0, -1.0 / n_load});
    discipline.add_point_load(load);
    MAST::NonlinearSystem sys;
    MAST::StructuralSystemInitialization init(sys, mesh);
    MAST::StructuralNonlinearAssemblyElemOperations ops;
    MAST::NonlinearImplicitAssembly assembly;
    assembly.set_discipline_and_system(discipline, init, ops);
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(0.01, 1.0);
    std::vector<Real> rho(mesh.n_elem());
    for (auto &r : rho) r = U(rng);
    assembly.set_simp(rho, 1e-9, 3.0);
    sys.opts.rtol = 1e-10;
    sys.solve(ops, assembly);
    REQUIRE(sys.last_report.status == MG_OK);
    REQUIRE(sys.last_report.relres <= 1e-10);
    MAST::ComplianceOutput compliance;
    assembly.calculate_output(sys.solution, false, compliance);
    MAST::Vector adjoint;
    sys.adjoint_solve(sys.solution, false, ops, compliance, assembly, adjoint);
    std::vector<std::unique_ptr<MAST::Parameter>> params;
    std::vector<const MAST::FunctionBase *> p_vec;
    for (int64_t e = 0; e < mesh.n_elem(); e += 37) {
        params.emplace_back(new MAST::Parameter(MAST::NonlinearImplicitAssembly::elem_param_name("rho", e), rho[e]));
        p_vec.push_back(params.back().get());
    }
    std::vector<Real> sens;
    assembly.calculate_output_adjoint_sensitivity_multiple_parameters_no_direct(sys.solution, false, adjoint, p_vec,
                                                                              ops, compliance, sens);
    // oracle
    or_simp_desc d{nx, ny, nz, 1.0, 1e-9, 0.3, 3.0, 0, ny, 1.0, 1e-12, 1000000};
    std::vector<double> u((size_t)3 * (nx + 1) * (ny + 1) * (nz + 1)), dc(mesh.n_elem());
    or_simp_report rep;
    REQUIRE(or_simp_solve(&d, rho.data(), u.data(), dc.data(), &rep) == 0);
    CHECK(compliance.output_total() == Approx(rep.compliance).epsilon(1e-10));
    for (size_t i = 0; i < p_vec.size(); i++) CHECK(sens[i] == Approx(dc[(size_t)i * 37]).epsilon(1e-9));
    // the general adjoint path (lambda . dR/drho_e) agrees with the compliance shortcut
    MAST::Vector dR;
    assembly.sensitivity_assemble(sys.solution, false, *p_vec[3], dR);
    Real s = 0;
    for (size_t k = 0; k < dR.size(); k++) s += adjoint(k) * dR(k);
    CHECK(s == Approx(sens[3]).epsilon(1e-9));
}

TEST_CASE("ks_stress_output_settings", "[cpu],[output]") {
    MAST::KSStressStrainOutput stress;
    stress.set_participating_elements_to_all();
    stress.set_aggregation_coefficients(8.0, 1.0, 0.5, 250.0);
    stress.set_stress_penalty(0.5);
    REQUIRE(stress.get_p_stress_val() == 8.0);
    REQUIRE(stress._sigma0 == 250.0);
    REQUIRE(stress.get_maximum_von_mises_stress() == 0.0);
    // the adjoint of the KS output is formed inside the library, not by adjoint_solve
    MAST::NonlinearSystem sys;
    MAST::NonlinearImplicitAssembly assembly;
    MAST::StructuralNonlinearAssemblyElemOperations ops;
    MAST::Vector X(3), adj;
    REQUIRE_THROWS(sys.adjoint_solve(X, false, ops, stress, assembly, adj));
}

// the reference's set_get_strain_type section
// (tests/property/mast_3d_isotropic_element_property_card.cpp:379-391)
// build_cube's boundary id b is libMesh side b of the boundary elements: the
// side's four nodes lie on that boundary's plane
TEST_CASE("hex8_boundary_sides", "[cpu],[mesh]") {
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_cube(mesh, 3, 2, 2, 0, 3, 0, 2, 0, 2);
    static const int side_nodes[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                         {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
    const int axis[6] = {2, 1, 0, 1, 0, 2};
    const double plane[6] = {0, 0, 3, 2, 0, 2};
    const size_t count[6] = {6, 6, 4, 6, 4, 6};
    for (int b = 0; b < 6; b++) {
        auto sides = mesh.boundary_sides(b);
        REQUIRE(sides.size() == count[b]);
        for (auto &es : sides) {
            REQUIRE(es.second == b);
            for (int i = 0; i < 4; i++) {
                const int64_t n = mesh.conn[(size_t)es.first * 8 + side_nodes[b][i]];
                const MAST::Point pt = mesh.point(n);
                const double c = axis[b] == 0 ? pt.x : axis[b] == 1 ? pt.y : pt.z;
                REQUIRE(c == plane[b]);
            }
        }
    }
}

TEST_CASE("section_strain_type", "[cpu],[property]") {
    MAST::Solid3DSectionElementPropertyCard section;
    REQUIRE(section.strain_type() == MAST::LINEAR_STRAIN);
    section.set_strain(MAST::LINEAR_STRAIN);
    REQUIRE(section.strain_type() == MAST::LINEAR_STRAIN);
    REQUIRE(!(section.strain_type() == MAST::NONLINEAR_STRAIN));
    section.set_strain(MAST::NONLINEAR_STRAIN);
    REQUIRE(section.strain_type() == MAST::NONLINEAR_STRAIN);
    REQUIRE(!(section.strain_type() == MAST::LINEAR_STRAIN));
}

// the section's NONLINEAR_STRAIN selects the Green-Lagrange element: a
// large-deflection cantilever solved by Newton through NonlinearSystem::solve,
// against a Newton iteration on the oracle's assembly; the compliance
// sensitivity from adjoint_solve + the general adjoint path against central
// differences of re-solved compliances
TEST_CASE("hex8_green_lagrange_cantilever", "[gpu],[structural],[3D],[nonlinear]") {
    const int nx = 6, ny = 2, nz = 2;
    const double P = 0.01;
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_cube(mesh, nx, ny, nz, 0, nx, 0, ny, 0, nz);
    MAST::Parameter E("E_param", 1.0), nu("nu_param", 0.3);
    MAST::ConstantFieldFunction E_f("E", E), nu_f("nu", nu);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(E_f);
    material.add(nu_f);
    MAST::Solid3DSectionElementPropertyCard section;
    section.set_material(material);
    section.set_strain(MAST::NONLINEAR_STRAIN);
    MAST::StructuralDiscipline discipline;
    discipline.set_property_for_subdomain(0, section);
    MAST::DirichletBoundaryCondition clamp;
    clamp.init(4, {0, 1, 2});
    discipline.add_dirichlet_bc(4, clamp);
    MAST::PointLoadCondition load(MAST::POINT_LOAD);
    std::vector<int64_t> tip;
    for (int64_t n : mesh.boundary_nodes(2))
        if (mesh.point(n).z == 0.0) tip.push_back(n);
    for (int64_t n : tip) load.add_node(n);
    load.set_load({0.0, 0.0, -P / tip.size()});
    discipline.add_point_load(load);
    MAST::NonlinearSystem sys;
    MAST::StructuralSystemInitialization init(sys, mesh);
    MAST::StructuralNonlinearAssemblyElemOperations ops;
    MAST::NonlinearImplicitAssembly assembly;
    assembly.set_discipline_and_system(discipline, init, ops);
    std::vector<Real> rho(mesh.n_elem());
    for (int64_t e = 0; e < mesh.n_elem(); e++) rho[e] = 0.7 + 0.3 * e / mesh.n_elem();
    assembly.set_simp(rho, 1e-9, 3.0);
    REQUIRE(assembly.physics() == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR);
    sys.opts.rtol = 1e-12;
    sys.opts.newton_rtol = 1e-12;
    sys.solve(ops, assembly);
    REQUIRE(sys.last_report.status == MG_OK);
    REQUIRE(sys.last_report.newton_iterations >= 3);

    // oracle Newton on the same system
    const int64_t nn = mesh.n_nodes(), n = 3 * nn, ne = mesh.n_elem();
    std::vector<int32_t> rowptr(n + 1);
    const int64_t nnz = or_csr_pattern(8, 3, nn, ne, mesh.conn.data(), rowptr.data(), nullptr);
    std::vector<int32_t> cols(nnz);
    or_csr_pattern(8, 3, nn, ne, mesh.conn.data(), rowptr.data(), cols.data());
    std::vector<double> Em(ne), dEm(ne), F(n, 0.0), u(n, 0.0), vals(nnz), R(n), du(n);
    for (int64_t e = 0; e < ne; e++) {
        const double rmin = 1e-9;
        Em[e] = rmin + (1 - rmin) * std::pow(rho[e], 3.0);
        dEm[e] = (1 - rmin) * 3.0 * rho[e] * rho[e];
    }
    std::vector<uint8_t> fixed(n, 0);
    for (int64_t nd : mesh.boundary_nodes(4))
        for (int c = 0; c < 3; c++) fixed[3 * nd + c] = 1;
    for (int64_t nd : tip) F[3 * nd + 2] -= P / tip.size();
    double r0 = -1;
    for (int it = 0; it < 40; it++) {
        REQUIRE(or_assemble_hex8_gl(nn, ne, mesh.coords.data(), mesh.conn.data(), Em.data(), 0.3, u.data(),
                                    F.data(), rowptr.data(), cols.data(), vals.data(), R.data(), fixed.data()) == 0);
        double rn = 0;
        for (double v : R) rn += v * v;
        rn = std::sqrt(rn);
        if (r0 < 0) r0 = rn;
        if (rn <= 1e-13 * r0) break;
        std::fill(du.begin(), du.end(), 0.0);
        double rr = 0;
        REQUIRE(or_pcg(n, rowptr.data(), cols.data(), vals.data(), R.data(), du.data(), 1e-14, 100000, &rr) >= 0);
        for (int64_t i = 0; i < n; i++) u[i] -= du[i];
    }
    double err = 0, umax = 0;
    for (int64_t i = 0; i < n; i++) {
        err = std::max(err, std::fabs(sys.solution(i) - u[i]));
        umax = std::max(umax, std::fabs(u[i]));
    }
    CHECK(err <= 1e-10 * umax);

    // compliance and its adjoint sensitivity (lambda from adjoint_solve)
    MAST::ComplianceOutput compliance;
    assembly.calculate_output(sys.solution, false, compliance);
    const double c0 = compliance.output_total();
    MAST::Vector adjoint;
    sys.adjoint_solve(sys.solution, false, ops, compliance, assembly, adjoint);
    std::vector<std::unique_ptr<MAST::Parameter>> params;
    std::vector<const MAST::FunctionBase *> p_vec;
    const int64_t probe[3] = {0, 11, ne - 1};
    for (int64_t e : probe) {
        params.emplace_back(new MAST::Parameter(MAST::NonlinearImplicitAssembly::elem_param_name("rho", e), rho[e]));
        p_vec.push_back(params.back().get());
    }
    std::vector<Real> sens;
    assembly.calculate_output_adjoint_sensitivity_multiple_parameters_no_direct(sys.solution, false, adjoint, p_vec,
                                                                              ops, compliance, sens);
    std::vector<double> dc(ne);
    double cc = 0;
    REQUIRE(mg_compliance(assembly.problem(), sys.solution.data(), &cc, dc.data()) == MG_OK);
    CHECK(cc == Approx(c0).epsilon(1e-14));
    const double h = 1e-5;
    for (int k = 0; k < 3; k++) {
        const int64_t e = probe[k];
        CHECK(sens[k] == Approx(dc[e]).epsilon(1e-9));
        double cpm[2];
        for (int s = 0; s < 2; s++) {
            std::vector<Real> r2 = rho;
            r2[e] += s == 0 ? h : -h;
            assembly.set_simp(r2, 1e-9, 3.0);
            sys.solution.zero();  // Newton's stop is relative to the initial residual: start from 0
            sys.solve(ops, assembly);
            REQUIRE(sys.last_report.status == MG_OK);
            assembly.calculate_output(sys.solution, false, compliance);
            cpm[s] = compliance.output_total();
        }
        CHECK(sens[k] == Approx((cpm[0] - cpm[1]) / (2 * h)).epsilon(1e-6));
    }
    assembly.set_simp(rho, 1e-9, 3.0);
}

// dR/drho_e from sensitivity_assemble against a central difference of the
// residual assembled by residual_and_jacobian
TEST_CASE("structural_sensitivity_assemble_matches_fd", "[gpu],[structural],[3D]") {
    const int nx = 4, ny = 3, nz = 2;
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_cube(mesh, nx, ny, nz, 0, nx, 0, ny, 0, nz);
    MAST::Parameter E("E_param", 1.0), nu("nu_param", 0.3);
    MAST::ConstantFieldFunction E_f("E", E), nu_f("nu", nu);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(E_f);
    material.add(nu_f);
    MAST::Solid3DSectionElementPropertyCard section;
    section.set_material(material);
    MAST::StructuralDiscipline discipline;
    discipline.set_property_for_subdomain(0, section);
    MAST::NonlinearSystem sys;
    MAST::StructuralSystemInitialization init(sys, mesh);
    MAST::StructuralNonlinearAssemblyElemOperations ops;
    MAST::NonlinearImplicitAssembly assembly;
    assembly.set_discipline_and_system(discipline, init, ops);
    std::vector<Real> rho(mesh.n_elem(), 0.6);
    assembly.set_simp(rho, 1e-9, 3.0);
    std::mt19937_64 rng(3);
    std::normal_distribution<double> N(0.0, 1.0);
    MAST::Vector X(3 * mesh.n_nodes());
    for (size_t i = 0; i < X.size(); i++) X(i) = 1e-2 * N(rng);
    const int64_t e = 7;
    MAST::Parameter p(MAST::NonlinearImplicitAssembly::elem_param_name("rho", e), rho[e]);
    MAST::Vector dR;
    assembly.sensitivity_assemble(X, false, p, dR);
    const double h = 1e-6;
    MAST::Vector Rp, Rm;
    rho[e] = 0.6 + h;
    assembly.set_simp(rho, 1e-9, 3.0);
    assembly.residual_and_jacobian(X, &Rp, nullptr, sys);
    rho[e] = 0.6 - h;
    assembly.set_simp(rho, 1e-9, 3.0);
    assembly.residual_and_jacobian(X, &Rm, nullptr, sys);
    double err = 0, ref = 0;
    for (size_t i = 0; i < X.size(); i++) {
        const double fd = (Rp(i) - Rm(i)) / (2 * h);
        err = std::max(err, std::fabs(fd - dR(i)));
        ref = std::max(ref, std::fabs(dR(i)));
    }
    REQUIRE(ref > 0);
    CHECK(err <= 1e-7 * ref);
}

// config 1 on a coarser grid: k(T) = k0 (1 + 0.01 T), q = 1 on [0.25, 0.75]^2,
// T = 0 at x = 0, convection h = 10, T_inf = 0 at x = 1
TEST_CASE("quad4_nonlinear_conduction", "[gpu],[heat],[2D]") {
    const int n = 40;
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_square(mesh, n, n, 0, 1, 0, 1);
    MAST::Parameter k("k_param", 1.0), beta("beta_param", 0.01), h("h_param", 1.0);
    MAST::ConstantFieldFunction k_f("k_th", k), b_f("k_beta", beta), h_f("h", h);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(k_f);
    material.add(b_f);
    MAST::Solid2DSectionElementPropertyCard section;
    section.set_material(material);
    section.add(h_f);
    MAST::HeatConductionDiscipline discipline;
    discipline.set_property_for_subdomain(0, section);
    MAST::DirichletBoundaryCondition left;
    left.init(3, {0});
    discipline.add_dirichlet_bc(3, left);
    MAST::Parameter hc("hc", 10.0), Tinf("Tinf", 0.0), q("q", 1.0);
    MAST::ConstantFieldFunction hc_f("convection_coeff", hc), Tinf_f("ambient_temperature", Tinf), q_f("heat_source", q);
    MAST::BoundaryConditionBase conv(MAST::CONVECTION_HEAT_FLUX), src(MAST::HEAT_SOURCE);
    conv.add(hc_f);
    conv.add(Tinf_f);
    src.add(q_f);
    discipline.add_side_load(1, conv);
    discipline.add_volume_load(1, src);
    MAST::NonlinearSystem sys;
    MAST::HeatConductionSystemInitialization init(sys, mesh);
    MAST::HeatConductionNonlinearAssemblyElemOperations ops;
    MAST::NonlinearImplicitAssembly assembly;
    std::vector<double> qe(mesh.n_elem(), 0.0);
    assembly._subdomain.assign(mesh.n_elem(), 0);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            const double xc = (i + 0.5) / n, yc = (j + 0.5) / n;
            if (xc > 0.25 && xc < 0.75 && yc > 0.25 && yc < 0.75) {
                assembly._subdomain[i + n * j] = 1;
                qe[i + n * j] = 1.0;
            }
        }
    assembly.set_discipline_and_system(discipline, init, ops);
    sys.opts.rtol = 1e-10;
    sys.opts.newton_rtol = 1e-10;
    sys.opts.consistent_jacobian = 1;
    sys.solve(ops, assembly);
    REQUIRE(sys.last_report.status == MG_OK);
    MAST::AverageTemperatureOutput Tbar;
    assembly.calculate_output(sys.solution, false, Tbar);
    or_heat_desc d{n, n, 1.0, 1.0, 1.0, 0.01, 1.0, 10.0, 0.0, 1e-12, 1e-12, 100000, 30, 1, 0};
    std::vector<double> T((size_t)(n + 1) * (n + 1)), s(mesh.n_elem(), 1.0), dq(mesh.n_elem());
    or_heat_report rep;
    REQUIRE(or_heat_solve(&d, s.data(), qe.data(), T.data(), dq.data(), &rep) == 0);
    CHECK(Tbar.output_total() == Approx(rep.mean_temperature).epsilon(1e-9));
    for (size_t i = 0; i < T.size(); i++) CHECK(sys.solution(i) == Approx(T[i]).epsilon(1e-8).margin(1e-12));
    // total dq/dk0 through the library's adjoint (mg_mean_temperature)
    mg_solve_opts o = sys.opts;
    double qv = 0, dk0 = 0;
    MAST::check(mg_mean_temperature(assembly.problem(), sys.solution.data(), &o, &qv, &dk0, nullptr), "mean T");
    CHECK(dk0 == Approx(rep.dq_dk0).epsilon(1e-7));
}

// MAST's direct-sensitivity route (NonlinearSystem::sensitivity_solve +
// AssemblyBase::calculate_output_direct_sensitivity) and the per-element plugin calls
// (init / set_elem_solution / elem_calculations / elem_sensitivity_calculations) of the
// structural element operations, against the oracle's element routines, the adjoint
// compliance sensitivity and re-solved central differences
TEST_CASE("structural_direct_sensitivity_and_element_plugin", "[gpu],[structural],[3D]") {
    const int nx = 8, ny = 4, nz = 4;
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_cube(mesh, nx, ny, nz, 0, nx, 0, ny, 0, nz);
    MAST::Parameter E("E_param", 1.0), nu("nu_param", 0.3);
    MAST::ConstantFieldFunction E_f("E", E), nu_f("nu", nu);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(E_f);
    material.add(nu_f);
    MAST::Solid3DSectionElementPropertyCard section;
    section.set_material(material);
    MAST::StructuralDiscipline discipline;
    discipline.set_property_for_subdomain(0, section);
    MAST::DirichletBoundaryCondition clamp;
    clamp.init(4, {0, 1, 2});
    discipline.add_dirichlet_bc(4, clamp);
    MAST::PointLoadCondition load(MAST::POINT_LOAD);
    int n_load = 0;
    for (int64_t n : mesh.boundary_nodes(2))
        if (mesh.point(n).z == 0.0) {
            load.add_node(n);
            n_load++;
        }
    load.set_load({0.0, 0.0, -1.0 / n_load});
    discipline.add_point_load(load);
    MAST::NonlinearSystem sys;
    MAST::StructuralSystemInitialization init(sys, mesh);
    MAST::StructuralNonlinearAssemblyElemOperations ops;
    MAST::NonlinearImplicitAssembly assembly;
    assembly.set_discipline_and_system(discipline, init, ops);
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<double> U(0.05, 1.0);
    std::vector<Real> rho(mesh.n_elem());
    for (auto &r : rho) r = U(rng);
    assembly.set_simp(rho, 1e-9, 3.0);
    sys.opts.rtol = 1e-13;
    sys.opts.max_iterations = 100000;
    sys.solve(ops, assembly);
    REQUIRE(sys.last_report.status == MG_OK);
    const MAST::Vector X = sys.solution;
    or_simp_desc d{nx, ny, nz, 1.0, 1e-9, 0.3, 3.0, 0, ny, 1.0, 1e-13, 1000000};
    std::vector<double> u_ref(X.size()), dc(mesh.n_elem()), Em(mesh.n_elem()), dEm(mesh.n_elem());
    or_simp_report rep;
    REQUIRE(or_simp_solve(&d, rho.data(), u_ref.data(), dc.data(), &rep) == 0);
    or_simp_modulus(&d, mesh.n_elem(), rho.data(), Em.data(), dEm.data());
    MAST::ComplianceOutput compliance;
    for (int64_t e : {0, 13, 77, 127}) {
        MAST::Parameter p(MAST::NonlinearImplicitAssembly::elem_param_name("rho", e), rho[e]);
        sys.sensitivity_solve(X, false, ops, assembly, p);
        const MAST::Vector dX = sys.get_sensitivity_solution();
        assembly.calculate_output_direct_sensitivity(X, false, &dX, false, p, compliance);
        // C = F.u: the direct route F . du/drho_e equals the adjoint -u_e^T dK_e/drho_e u_e
        CHECK(compliance.output_sensitivity_total(p) == Approx(dc[e]).epsilon(1e-8));
        // without dX/dp the partial derivative: the compliance has no explicit density term
        assembly.calculate_output_direct_sensitivity(X, false, nullptr, false, p, compliance);
        CHECK(compliance.output_sensitivity_total(p) == 0.0);
        if (e == 77) {
            // du/drho_e against a central difference of re-solved displacements
            const double h = 1e-5;
            MAST::Vector up, um;
            rho[e] += h;
            assembly.set_simp(rho, 1e-9, 3.0);
            sys.solve(ops, assembly);
            up = sys.solution;
            rho[e] -= 2 * h;
            assembly.set_simp(rho, 1e-9, 3.0);
            sys.solve(ops, assembly);
            um = sys.solution;
            rho[e] += h;
            assembly.set_simp(rho, 1e-9, 3.0);
            double err = 0, ref = 0;
            for (size_t i = 0; i < X.size(); i++) {
                err = std::max(err, std::fabs((up(i) - um(i)) / (2 * h) - dX(i)));
                ref = std::max(ref, std::fabs(dX(i)));
            }
            REQUIRE(ref > 0);
            CHECK(err <= 1e-6 * ref);
        }
    }
    // the per-element plugin calls, as MAST's own assembly loop makes them
    MAST::Vector R(X.size());
    std::vector<int64_t> fixed_rows;
    for (int64_t e = 0; e < mesh.n_elem(); e++) {
        MAST::GeomElem geom;
        geom.init(e, init);
        ops.init(geom);
        const int32_t *en = &mesh.conn[(size_t)e * 8];
        MAST::RealVectorX sol(24);
        double Xe[24], ue[24];
        for (int a = 0; a < 8; a++)
            for (int c = 0; c < 3; c++) {
                sol[c * 8 + a] = X((size_t)en[a] * 3 + c);
                ue[c * 8 + a] = sol[c * 8 + a];
                Xe[a * 3 + c] = mesh.coords[(size_t)en[a] * 3 + c];
            }
        ops.set_elem_solution(sol);
        MAST::RealVectorX vec;
        MAST::RealMatrixX mat;
        ops.elem_calculations(true, vec, mat);
        double f_ref[24], K_ref[576];
        REQUIRE(or_hex8_internal(Xe, Em[e], 0.3, ue, f_ref, K_ref) == 0);
        double ek = 0, rk = 0, ef = 0, rf = 0;
        for (int i = 0; i < 24; i++) {
            ef = std::max(ef, std::fabs(vec[i] - f_ref[i]));
            rf = std::max(rf, std::fabs(f_ref[i]));
            for (int j = 0; j < 24; j++) {
                ek = std::max(ek, std::fabs(mat(i, j) - K_ref[i * 24 + j]));
                rk = std::max(rk, std::fabs(K_ref[i * 24 + j]));
            }
        }
        CHECK(ek <= 1e-12 * rk);
        CHECK(ef <= 1e-12 * rf);
        if (e % 29 == 0) {
            MAST::Parameter own(MAST::NonlinearImplicitAssembly::elem_param_name("rho", e), rho[e]);
            MAST::Parameter other(MAST::NonlinearImplicitAssembly::elem_param_name("rho", (e + 1) % mesh.n_elem()), 0.5);
            MAST::RealVectorX dvec, zvec;
            ops.elem_sensitivity_calculations(own, dvec);
            ops.elem_sensitivity_calculations(other, zvec);
            double df_ref[24];
            REQUIRE(or_hex8_internal_sens(Xe, dEm[e], 0.3, ue, df_ref) == 0);
            double ed = 0, rd = 0, ez = 0;
            for (int i = 0; i < 24; i++) {
                ed = std::max(ed, std::fabs(dvec[i] - df_ref[i]));
                rd = std::max(rd, std::fabs(df_ref[i]));
                ez = std::max(ez, std::fabs(zvec[i]));
            }
            CHECK(ed <= 1e-12 * rd);
            CHECK(ez == 0.0);
        }
        ops.clear_elem();
        for (int a = 0; a < 8; a++)
            for (int c = 0; c < 3; c++) R((size_t)en[a] * 3 + c) += vec[c * 8 + a];
    }
    // assembled from the plugin calls: R = f_int - F equals residual_and_jacobian's R on
    // the free dofs (at the converged solution both are ~0 relative to f_int; compare at
    // a perturbed state instead would need a second loop, so compare f_int - F directly)
    MAST::Vector F = assembly.load_vector(), R_lib;
    assembly.residual_and_jacobian(X, &R_lib, nullptr, sys);
    double err = 0, ref = 0;
    for (size_t i = 0; i < X.size(); i++) {
        ref = std::max(ref, std::fabs(R(i)));
        if (F(i) == 0.0 && R_lib(i) == X(i)) continue;  // constrained row: R_d = X_d
        err = std::max(err, std::fabs((R(i) - F(i)) - R_lib(i)));
    }
    REQUIRE(ref > 0);
    CHECK(err <= 1e-10 * ref);
}

// forward sensitivity of the nonlinear conduction solution to k0 and the mean
// temperature's direct sensitivity, against the adjoint route of mg_mean_temperature;
// the heat element plugin calls against the oracle's element routines
TEST_CASE("heat_direct_sensitivity_and_element_plugin", "[gpu],[heat],[2D]") {
    const int n = 20;
    MAST::Mesh mesh;
    MAST::MeshTools::Generation::build_square(mesh, n, n, 0, 1, 0, 1);
    MAST::Parameter k("k_param", 1.0), beta("beta_param", 0.01), h("h_param", 1.0);
    MAST::ConstantFieldFunction k_f("k_th", k), b_f("k_beta", beta), h_f("h", h);
    MAST::IsotropicMaterialPropertyCard material;
    material.add(k_f);
    material.add(b_f);
    MAST::Solid2DSectionElementPropertyCard section;
    section.set_material(material);
    section.add(h_f);
    MAST::HeatConductionDiscipline discipline;
    discipline.set_property_for_subdomain(0, section);
    MAST::DirichletBoundaryCondition left;
    left.init(3, {0});
    discipline.add_dirichlet_bc(3, left);
    MAST::Parameter hc("hc", 10.0), Tinf("Tinf", 0.0), q("q", 1.0);
    MAST::ConstantFieldFunction hc_f("convection_coeff", hc), Tinf_f("ambient_temperature", Tinf), q_f("heat_source", q);
    MAST::BoundaryConditionBase conv(MAST::CONVECTION_HEAT_FLUX), src(MAST::HEAT_SOURCE);
    conv.add(hc_f);
    conv.add(Tinf_f);
    src.add(q_f);
    discipline.add_side_load(1, conv);
    discipline.add_volume_load(-1, src);
    MAST::NonlinearSystem sys;
    MAST::HeatConductionSystemInitialization init(sys, mesh);
    MAST::HeatConductionNonlinearAssemblyElemOperations ops;
    MAST::NonlinearImplicitAssembly assembly;
    assembly.set_discipline_and_system(discipline, init, ops);
    sys.opts.rtol = 1e-13;
    sys.opts.newton_rtol = 1e-13;
    sys.opts.consistent_jacobian = 1;
    sys.opts.krylov = MG_KRYLOV_BICGSTAB;
    sys.solve(ops, assembly);
    REQUIRE(sys.last_report.status == MG_OK);
    const MAST::Vector T = sys.solution;
    MAST::Parameter k0p("k0", 1.0);
    sys.sensitivity_solve(T, false, ops, assembly, k0p);
    const MAST::Vector dT = sys.get_sensitivity_solution();
    MAST::AverageTemperatureOutput Tbar;
    assembly.calculate_output_direct_sensitivity(T, false, &dT, false, k0p, Tbar);
    mg_solve_opts o = sys.opts;
    double qv = 0, dk0 = 0;
    MAST::check(mg_mean_temperature(assembly.problem(), T.data(), &o, &qv, &dk0, nullptr), "mean T");
    CHECK(Tbar.output_sensitivity_total(k0p) == Approx(dk0).epsilon(1e-8));
    // element plugin: conduction + convection + source of each element at T
    for (int64_t e = 0; e < mesh.n_elem(); e++) {
        MAST::GeomElem geom;
        geom.init(e, init);
        ops.init(geom);
        const int32_t *en = &mesh.conn[(size_t)e * 4];
        MAST::RealVectorX sol(4);
        double Xe[8];
        for (int a = 0; a < 4; a++) {
            sol[a] = T((size_t)en[a]);
            Xe[a * 2] = mesh.coords[(size_t)en[a] * 2];
            Xe[a * 2 + 1] = mesh.coords[(size_t)en[a] * 2 + 1];
        }
        ops.set_elem_solution(sol);
        MAST::RealVectorX vec;
        MAST::RealMatrixX mat;
        ops.elem_calculations(true, vec, mat);
        double f[4], K[16], fc[4] = {0, 0, 0, 0}, Kc[16] = {0}, fs[4];
        REQUIRE(or_quad4_heat_internal(Xe, 1.0, 0.01, 1.0, 1.0, sol.data(), 1, f, K) == 0);
        const int i = (int)(e % n);
        if (i == n - 1) or_quad4_heat_convection(Xe, 1, 10.0, 0.0, 1.0, sol.data(), fc, Kc);
        or_quad4_heat_source(Xe, 1.0, 1.0, fs);
        double ef = 0, rf = 0, ek = 0, rk = 0;
        for (int a = 0; a < 4; a++) {
            const double fr = f[a] + fc[a] + fs[a];
            ef = std::max(ef, std::fabs(vec[a] - fr));
            rf = std::max(rf, std::fabs(fr));
            for (int b = 0; b < 4; b++) {
                ek = std::max(ek, std::fabs(mat(a, b) - (K[a * 4 + b] + Kc[a * 4 + b])));
                rk = std::max(rk, std::fabs(K[a * 4 + b] + Kc[a * 4 + b]));
            }
        }
        CHECK(ef <= 1e-12 * rf);
        CHECK(ek <= 1e-12 * rk);
        if (e % 37 == 0) {
            // d f_e / d k0 = int grad(phi) (1 + beta T) h grad(T)
            MAST::RealVectorX dvec;
            ops.elem_sensitivity_calculations(k0p, dvec);
            double df[4];
            REQUIRE(or_quad4_heat_internal_sens(Xe, 1.0, 0.01, 1.0, sol.data(), df) == 0);
            double ed = 0, rd = 0;
            for (int a = 0; a < 4; a++) {
                ed = std::max(ed, std::fabs(dvec[a] - df[a]));
                rd = std::max(rd, std::fabs(df[a]));
            }
            CHECK(ed <= 1e-12 * std::max(rd, 1e-300));
        }
        ops.clear_elem();
    }
}

MINI_CATCH_MAIN
