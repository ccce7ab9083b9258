// mast_api.hpp -- C++ host mirror of the part of MAST's API that sits on the
// GPU hot path, with light types instead of libMesh/Eigen/PETSc, forwarding
// to the C ABI in mastgpu.h.  Header-only; link libmastgpu.so.
//
// Mirrored (same class and method names, same argument meaning, same error
// behaviour: MAST reports misuse through libmesh_error_msg, here a
// MAST::Error exception carrying the library's status):
//   MAST::Parameter, MAST::FunctionBase, MAST::FieldFunction<T>,
//   MAST::ConstantFieldFunction                 src/base/parameter.h, field_function_base.h,
//                                               constant_field_function.h
//   MAST::IsotropicMaterialPropertyCard          src/property_cards/isotropic_material_property_card.h
//     (stiffness_matrix(dim, plane_strain), conductance_matrix(dim): the
//      formulas of isotropic_material_property_card.cpp:395-567, 716-748)
//   MAST::Solid3DSectionElementPropertyCard,
//   MAST::Solid2DSectionElementPropertyCard      src/property_cards/solid_*d_section_element_property_card.h
//   MAST::DirichletBoundaryCondition::init(bid, vars)   src/boundary_condition/dirichlet_boundary_condition.h:67
//   MAST::PointLoadCondition(POINT_LOAD)::add_node, "load"  src/boundary_condition/point_load_condition.h
//   MAST::BoundaryConditionBase(CONVECTION_HEAT_FLUX / HEAT_SOURCE / SURFACE_PRESSURE / HEAT_FLUX)
//                                                src/base/boundary_condition_base.h:29-51
//   MAST::PhysicsDisciplineBase::add_dirichlet_bc / add_point_load / add_side_load /
//     add_volume_load / set_property_for_subdomain   src/base/physics_discipline_base.h:94-206
//   MAST::StructuralSystemInitialization, MAST::HeatConductionSystemInitialization
//   MAST::StructuralNonlinearAssemblyElemOperations,
//   MAST::HeatConductionNonlinearAssemblyElemOperations
//   MAST::NonlinearImplicitAssembly::residual_and_jacobian(X, R, J, S)
//                                               src/base/nonlinear_implicit_assembly.h:99-104
//     ::sensitivity_assemble(X, localize, f, rhs, close)   src/base/assembly_base.h:245-252
//     ::calculate_output(X, localize, output)             src/base/assembly_base.h:257-260
//     ::calculate_output_adjoint_sensitivity_multiple_parameters_no_direct(...)
//                                               src/base/assembly_base.h:313-321
//   MAST::NonlinearSystem::solve(elem_ops, assembly), ::adjoint_solve(...),
//     ::sensitivity_solve(X, localize, elem_ops, assembly, p)  src/base/nonlinear_system.h:133-155
//   MAST::NonlinearImplicitAssembly::calculate_output_derivative(X, localize, output, dq_dX),
//     ::calculate_output_direct_sensitivity(X, localize, dXdp, localize_sens, p, output)
//                                               src/base/assembly_base.h:266-290
//   MAST::AssemblyElemOperations::set_assembly / init(GeomElem) / set_elem_solution /
//     clear_elem, MAST::NonlinearImplicitAssemblyElemOperations::elem_calculations(if_jac,
//     vec, mat) / elem_sensitivity_calculations(f, vec)
//                                               src/base/assembly_elem_operation.h:40-176,
//                                               nonlinear_implicit_assembly_elem_operations.h:50-105
//   MAST::ComplianceOutput                       src/elasticity/compliance_output.h
//   libMesh::MeshTools::Generation::build_cube / build_square (unit-spaced
//   HEX8/QUAD4 grids, libMesh node numbering and boundary ids) -> MAST::Mesh
//
// Global vectors are MAST::Vector (dof = dpn * node + component, the library's
// numbering; MAST's DofMap numbering is mapped by the integrating adapter).
#pragma once

#include <cmath>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mastgpu.h"

namespace MAST {

typedef double Real;

// ------------------------------------------------------------------ light types
class Error : public std::runtime_error {
public:
    Error(int status, const std::string &where)
        : std::runtime_error(where + ": " + mg_status_string(status) + " (" + mg_last_error() + ")"),
          status(status) {}
    int status;
};

inline void check(int status, const char *where) {
    if (status != MG_OK) throw Error(status, where);
}

struct Point {
    Real x = 0, y = 0, z = 0;
    Point(Real a = 0, Real b = 0, Real c = 0) : x(a), y(b), z(c) {}
};

typedef std::vector<Real> RealVectorX;

class RealMatrixX {
public:
    RealMatrixX(int r = 0, int c = 0) : _r(r), _c(c), _v((size_t)r * c, 0.0) {}
    static RealMatrixX Zero(int r, int c) { return RealMatrixX(r, c); }
    Real &operator()(int i, int j) { return _v[(size_t)i * _c + j]; }
    Real operator()(int i, int j) const { return _v[(size_t)i * _c + j]; }
    int rows() const { return _r; }
    int cols() const { return _c; }
    const std::vector<Real> &data() const { return _v; }

private:
    int _r, _c;
    std::vector<Real> _v;
};

// global vector (stands in for libMesh::NumericVector<Real>)
class Vector {
public:
    explicit Vector(size_t n = 0) : _v(n, 0.0) {}
    size_t size() const { return _v.size(); }
    Real &operator()(size_t i) { return _v[i]; }
    Real operator()(size_t i) const { return _v[i]; }
    Real *data() { return _v.data(); }
    const Real *data() const { return _v.data(); }
    void zero() { std::fill(_v.begin(), _v.end(), 0.0); }
    void close() {}
    void resize(size_t n) { _v.assign(n, 0.0); }
    Real l2_norm() const {
        Real s = 0;
        for (Real x : _v) s += x * x;
        return std::sqrt(s);
    }

private:
    std::vector<Real> _v;
};

// CSR matrix (stands in for libMesh::SparseMatrix<Real>)
struct SparseMatrix {
    int64_t n = 0;
    std::vector<int32_t> rowptr, cols;
    std::vector<Real> vals;
    void close() {}
    Real operator()(int64_t i, int64_t j) const {
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; k++)
            if (cols[k] == j) return vals[k];
        return 0.0;
    }
};

// ------------------------------------------------------------------ functions
class FunctionBase {
public:
    explicit FunctionBase(const std::string &nm) : _name(nm) {}
    virtual ~FunctionBase() {}
    const std::string &name() const { return _name; }

protected:
    std::string _name;
};

class Parameter : public FunctionBase {
public:
    Parameter(const std::string &nm, Real v) : FunctionBase(nm), _val(v) {}
    Real operator()() const { return _val; }
    Parameter &operator=(Real v) {
        _val = v;
        return *this;
    }

private:
    Real _val;
};

template <class T>
class FieldFunction : public FunctionBase {
public:
    explicit FieldFunction(const std::string &nm) : FunctionBase(nm) {}
    virtual void operator()(const Point &p, Real t, T &v) const = 0;
    virtual void derivative(const FunctionBase &f, const Point &p, Real t, T &v) const = 0;
};

class ConstantFieldFunction : public FieldFunction<Real> {
public:
    ConstantFieldFunction(const std::string &nm, const Parameter &p) : FieldFunction<Real>(nm), _p(&p) {}
    void operator()(const Point &, Real, Real &v) const override { v = (*_p)(); }
    void derivative(const FunctionBase &f, const Point &, Real, Real &v) const override {
        v = (&f == _p) ? 1.0 : 0.0;
    }
    const Parameter &parameter() const { return *_p; }

private:
    const Parameter *_p;
};

// a matrix-valued property of the material card
class MatrixFunction : public FieldFunction<RealMatrixX> {
public:
    typedef RealMatrixX (*Eval)(const std::map<std::string, Real> &, int, bool);
    MatrixFunction(const std::string &nm, std::map<std::string, const FieldFunction<Real> *> props, int dim,
                   bool flag, Eval fn)
        : FieldFunction<RealMatrixX>(nm), _props(props), _dim(dim), _flag(flag), _fn(fn) {}
    void operator()(const Point &p, Real t, RealMatrixX &m) const override {
        std::map<std::string, Real> v;
        for (auto &kv : _props) (*kv.second)(p, t, v[kv.first]);
        m = _fn(v, _dim, _flag);
    }
    // central difference in the named parameter is not needed: the formulas are
    // linear in E and k, so d/dp = (value at dE/dp, dk/dp) with nu held
    void derivative(const FunctionBase &f, const Point &p, Real t, RealMatrixX &m) const override {
        std::map<std::string, Real> v;
        for (auto &kv : _props) {
            Real val;
            (*kv.second)(p, t, val);
            Real dv;
            kv.second->derivative(f, p, t, dv);
            v[kv.first] = (kv.first == "nu") ? val : dv;
            if (kv.first == "nu" && dv != 0.0)
                throw std::runtime_error("derivative with respect to nu is not provided");
        }
        m = _fn(v, _dim, _flag);
    }

private:
    std::map<std::string, const FieldFunction<Real> *> _props;
    int _dim;
    bool _flag;
    Eval _fn;
};

// ------------------------------------------------------------------ property cards
class MaterialPropertyCardBase {
public:
    virtual ~MaterialPropertyCardBase() {}
    void add(const FieldFunction<Real> &f) { _f[f.name()] = &f; }
    bool contains(const std::string &nm) const { return _f.count(nm) != 0; }
    template <class T>
    const T &get(const std::string &nm) const {
        auto it = _f.find(nm);
        if (it == _f.end()) throw std::runtime_error("property card has no function " + nm);
        return dynamic_cast<const T &>(*it->second);
    }
    Real value(const std::string &nm) const {
        Real v;
        get<FieldFunction<Real>>(nm)(Point(), 0.0, v);
        return v;
    }

protected:
    std::map<std::string, const FieldFunction<Real> *> _f;
};

class IsotropicMaterialPropertyCard : public MaterialPropertyCardBase {
public:
    // isotropic_material_property_card.cpp:395-426 (2D plane stress / strain),
    // :512-528 (3D): Voigt [xx, yy, zz, xy, yz, zx], engineering shear
    static RealMatrixX stiffness_formula(const std::map<std::string, Real> &v, int dim, bool plane_strain) {
        const Real E = v.at("E"), nu = v.at("nu");
        if (dim == 3) {
            RealMatrixX C(6, 6);
            const Real a = E * (1 - nu) / (1 - nu - 2 * nu * nu), b = E * nu / (1 - nu - 2 * nu * nu);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) C(i, j) = (i == j) ? a : b;
            for (int i = 3; i < 6; i++) C(i, i) = E / 2.0 / (1 + nu);
            return C;
        }
        if (dim == 2) {
            RealMatrixX C(3, 3);
            if (!plane_strain) {
                C(0, 0) = C(1, 1) = E / (1 - nu * nu);
                C(0, 1) = C(1, 0) = E * nu / (1 - nu * nu);
            } else {
                const Real f = E / (1 + nu) / (1 - 2 * nu);
                C(0, 0) = C(1, 1) = f * (1 - nu);
                C(0, 1) = C(1, 0) = f * nu;
            }
            C(2, 2) = E / 2.0 / (1 + nu);
            return C;
        }
        RealMatrixX C(2, 2);
        C(0, 0) = E;
        C(1, 1) = E / 2.0 / (1 + nu);
        return C;
    }
    // :716-748: k I
    static RealMatrixX conductance_formula(const std::map<std::string, Real> &v, int dim, bool) {
        RealMatrixX K(dim, dim);
        for (int i = 0; i < dim; i++) K(i, i) = v.at("k_th");
        return K;
    }
    const FieldFunction<RealMatrixX> &stiffness_matrix(int dim, bool plane_strain = false) {
        std::map<std::string, const FieldFunction<Real> *> p = {{"E", &get<FieldFunction<Real>>("E")},
                                                                {"nu", &get<FieldFunction<Real>>("nu")}};
        _m.emplace_back(new MatrixFunction("StiffnessMatrix", p, dim, plane_strain, &stiffness_formula));
        return *_m.back();
    }
    const FieldFunction<RealMatrixX> &conductance_matrix(int dim) {
        std::map<std::string, const FieldFunction<Real> *> p = {{"k_th", &get<FieldFunction<Real>>("k_th")}};
        _m.emplace_back(new MatrixFunction("ConductanceMatrix", p, dim, false, &conductance_formula));
        return *_m.back();
    }

private:
    std::vector<std::unique_ptr<MatrixFunction>> _m;
};

// ElementPropertyCardBase's strain type (element_property_card_base.h:36-41,
// set_strain / strain_type :183-194): NONLINEAR_STRAIN selects the Green-Lagrange
// branch of the 3D solid element
enum StrainType { LINEAR_STRAIN, NONLINEAR_STRAIN };

class ElementPropertyCardBase : public MaterialPropertyCardBase {
public:
    void set_strain(StrainType strain) { _strain = strain; }
    StrainType strain_type() const { return _strain; }
    void set_material(const IsotropicMaterialPropertyCard &m) { _mat = &m; }
    const IsotropicMaterialPropertyCard &get_material() const {
        if (!_mat) throw std::runtime_error("element property card has no material");
        return *_mat;
    }
    virtual int dim() const = 0;

private:
    const IsotropicMaterialPropertyCard *_mat = nullptr;
    StrainType _strain = LINEAR_STRAIN;
};

class Solid3DSectionElementPropertyCard : public ElementPropertyCardBase {
public:
    int dim() const override { return 3; }
};

class Solid2DSectionElementPropertyCard : public ElementPropertyCardBase {
public:
    int dim() const override { return 2; }
};

// ------------------------------------------------------------------ mesh
enum ElemType { HEX8, QUAD4 };

// unit-spaced structured grid with libMesh's numbering: node (i, j, k) is
// i + (nx+1)(j + (ny+1) k); boundary ids of build_cube: 0 z=0, 1 y=0, 2 x=max,
// 3 y=max, 4 x=0, 5 z=max; of build_square: 0 y=0, 1 x=max, 2 y=max, 3 x=0
class Mesh {
public:
    ElemType type = HEX8;
    int nx = 0, ny = 0, nz = 0;  // structured-grid dims (0: an unstructured mesh)
    std::vector<Real> coords;    // n_nodes x dim
    std::vector<int32_t> conn;   // n_elems x npe, libMesh local order
    std::map<int, std::vector<int64_t>> node_boundary;  // unstructured meshes: nodes per boundary id
    int dim() const { return type == HEX8 ? 3 : 2; }
    int64_t n_nodes() const { return (int64_t)coords.size() / dim(); }
    int64_t n_elem() const { return (int64_t)conn.size() / (type == HEX8 ? 8 : 4); }
    Point point(int64_t n) const {
        return type == HEX8 ? Point(coords[3 * n], coords[3 * n + 1], coords[3 * n + 2])
                            : Point(coords[2 * n], coords[2 * n + 1]);
    }
    // nodes on a boundary id
    std::vector<int64_t> boundary_nodes(int bid) const {
        std::vector<int64_t> out;
        if (nx == 0) {  // unstructured: the boundary node sets read with the mesh
            auto it = node_boundary.find(bid);
            return it == node_boundary.end() ? out : it->second;
        }
        const int NX = nx + 1, NY = ny + 1, NZ = type == HEX8 ? nz + 1 : 1;
        for (int k = 0; k < NZ; k++)
            for (int j = 0; j < NY; j++)
                for (int i = 0; i < NX; i++) {
                    bool on;
                    if (type == HEX8) {
                        const bool b[6] = {k == 0, j == 0, i == nx, j == ny, i == 0, k == nz};
                        on = bid >= 0 && bid < 6 && b[bid];
                    } else {
                        const bool b[4] = {j == 0, i == nx, j == ny, i == 0};
                        on = bid >= 0 && bid < 4 && b[bid];
                    }
                    if (on) out.push_back(i + (int64_t)NX * (j + (int64_t)NY * k));
                }
        return out;
    }
    // element sides on a boundary id of a structured grid (libMesh side numbers: QUAD4
    // 0..3; HEX8 0..5, where build_cube's boundary id b is side b of the boundary elements)
    std::vector<std::pair<int32_t, int32_t>> boundary_sides(int bid) const {
        std::vector<std::pair<int32_t, int32_t>> out;
        if (type == HEX8) {
            if (nx == 0) return out;
            for (int k = 0; k < nz; k++)
                for (int j = 0; j < ny; j++)
                    for (int i = 0; i < nx; i++) {
                        const bool on[6] = {k == 0, j == 0, i == nx - 1, j == ny - 1, i == 0, k == nz - 1};
                        if (bid >= 0 && bid < 6 && on[bid]) out.push_back({i + nx * (j + ny * k), bid});
                    }
            return out;
        }
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const int32_t e = i + nx * j;
                if (bid == 0 && j == 0) out.push_back({e, 0});
                if (bid == 1 && i == nx - 1) out.push_back({e, 1});
                if (bid == 2 && j == ny - 1) out.push_back({e, 2});
                if (bid == 3 && i == 0) out.push_back({e, 3});
            }
        return out;
    }
};

namespace MeshTools {
namespace Generation {
inline void build_cube(Mesh &m, int nx, int ny, int nz, Real x0, Real x1, Real y0, Real y1, Real z0, Real z1) {
    m = Mesh();
    m.type = HEX8;
    m.nx = nx; m.ny = ny; m.nz = nz;
    const int NX = nx + 1, NY = ny + 1, NZ = nz + 1;
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++) {
                m.coords.push_back(x0 + (x1 - x0) * i / nx);
                m.coords.push_back(y0 + (y1 - y0) * j / ny);
                m.coords.push_back(z0 + (z1 - z0) * k / nz);
            }
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const int32_t n0 = i + NX * (j + NY * k);
                const int32_t c[8] = {n0, n0 + 1, n0 + 1 + NX, n0 + NX,
                                      n0 + NX * NY, n0 + 1 + NX * NY, n0 + 1 + NX + NX * NY, n0 + NX + NX * NY};
                m.conn.insert(m.conn.end(), c, c + 8);
            }
}
inline void build_square(Mesh &m, int nx, int ny, Real x0, Real x1, Real y0, Real y1) {
    m = Mesh();
    m.type = QUAD4;
    m.nx = nx; m.ny = ny; m.nz = 0;
    const int NX = nx + 1;
    for (int j = 0; j <= ny; j++)
        for (int i = 0; i <= nx; i++) {
            m.coords.push_back(x0 + (x1 - x0) * i / nx);
            m.coords.push_back(y0 + (y1 - y0) * j / ny);
        }
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const int32_t n0 = i + NX * j;
            const int32_t c[4] = {n0, n0 + 1, n0 + 1 + NX, n0 + NX};
            m.conn.insert(m.conn.end(), c, c + 4);
        }
}
}  // namespace Generation
}  // namespace MeshTools

// MAST::NastranIO (src/mesh/nastran_io.h / .cpp): reads a Nastran bulk data
// deck into the mesh -- GRID nodes (ascending id), CHEXA / CQUAD4 elements
// (ascending id), every SPC node as boundary id 1 -- through mg_bdf_read
// instead of pyNastran
class NastranIO {
public:
    explicit NastranIO(Mesh &mesh, bool python_preinitialized = false) : _mesh(mesh) { (void)python_preinitialized; }
    void read(const std::string &filename) {
        mg_bdf_mesh *h = nullptr;
        check(mg_bdf_read(filename.c_str(), &h), "NastranIO::read");
        int64_t nn = 0, ne = 0, nspc = 0;
        int32_t npe = 0;
        mg_bdf_sizes(h, &nn, &ne, &npe);
        std::vector<double> xyz((size_t)nn * 3);
        std::vector<int64_t> gids((size_t)nn), eids((size_t)ne);
        Mesh m;
        m.type = npe == 8 ? HEX8 : QUAD4;
        m.conn.resize((size_t)ne * npe);
        mg_bdf_nodes(h, xyz.data(), gids.data());
        mg_bdf_elements(h, m.conn.data(), eids.data(), nullptr);
        mg_bdf_constraints(h, 6, nullptr, &nspc);
        std::vector<int64_t> spc((size_t)nspc);
        mg_bdf_constraints(h, 6, spc.data(), &nspc);
        mg_bdf_destroy(h);
        for (int64_t n = 0; n < nn; n++)
            for (int k = 0; k < m.dim(); k++) m.coords.push_back(xyz[3 * n + k]);
        std::set<int64_t> spc_nodes;
        for (int64_t d : spc) spc_nodes.insert(d / 6);
        if (!spc_nodes.empty()) m.node_boundary[1].assign(spc_nodes.begin(), spc_nodes.end());
        _node_map.clear();
        _elem_map.clear();
        for (int64_t n = 0; n < nn; n++) _node_map[(uint64_t)gids[n]] = n;
        for (int64_t e = 0; e < ne; e++) _elem_map[(uint64_t)eids[e]] = e;
        _mesh = m;
    }
    // Nastran id -> mesh node / element index
    std::map<uint64_t, int64_t> get_nastran_to_libmesh_node_map() const { return _node_map; }
    std::map<uint64_t, int64_t> get_nastran_to_libmesh_elem_map() const { return _elem_map; }

private:
    Mesh &_mesh;
    std::map<uint64_t, int64_t> _node_map, _elem_map;
};

// ------------------------------------------------------------------ boundary conditions
enum BoundaryConditionType { POINT_LOAD, DIRICHLET, CONVECTION_HEAT_FLUX, HEAT_SOURCE, SURFACE_PRESSURE, HEAT_FLUX };

class BoundaryConditionBase : public MaterialPropertyCardBase {
public:
    explicit BoundaryConditionBase(BoundaryConditionType t) : _type(t) {}
    BoundaryConditionType type() const { return _type; }

private:
    BoundaryConditionType _type;
};

class DirichletBoundaryCondition : public BoundaryConditionBase {
public:
    DirichletBoundaryCondition() : BoundaryConditionBase(DIRICHLET) {}
    // homogeneous constraint of the listed system variables on boundary `bid`
    void init(int bid, const std::vector<unsigned int> &constrained_vars) {
        _bid = bid;
        _vars = constrained_vars;
    }
    int boundary_id() const { return _bid; }
    const std::vector<unsigned int> &vars() const { return _vars; }

private:
    int _bid = -1;
    std::vector<unsigned int> _vars;
};

// the load vector: one value per system variable ("load" function of MAST's
// PointLoadCondition; here a constant vector)
class PointLoadCondition : public BoundaryConditionBase {
public:
    explicit PointLoadCondition(BoundaryConditionType t) : BoundaryConditionBase(t) {
        if (t != POINT_LOAD) throw std::runtime_error("PointLoadCondition needs POINT_LOAD");
    }
    void add_node(int64_t node) { _nodes.insert(node); }
    const std::set<int64_t> &get_nodes() const { return _nodes; }
    void set_load(const RealVectorX &v) { _load = v; }
    const RealVectorX &load() const { return _load; }

private:
    std::set<int64_t> _nodes;
    RealVectorX _load;
};

// ------------------------------------------------------------------ disciplines
class PhysicsDisciplineBase {
public:
    virtual ~PhysicsDisciplineBase() {}
    void add_dirichlet_bc(int bid, DirichletBoundaryCondition &bc) { _dir.push_back(&bc); (void)bid; }
    void add_point_load(PointLoadCondition &l) { _pl.push_back(&l); }
    void add_side_load(int bid, BoundaryConditionBase &bc) { _side.push_back({bid, &bc}); }
    // per-element source q_e: element e of `elems` carries the "heat_source" value
    void add_volume_load(int sid, BoundaryConditionBase &bc) { _vol.push_back({sid, &bc}); }
    void set_property_for_subdomain(int sid, const ElementPropertyCardBase &p) { _prop = &p; (void)sid; }
    const ElementPropertyCardBase &property() const {
        if (!_prop) throw std::runtime_error("no element property card set");
        return *_prop;
    }
    std::vector<DirichletBoundaryCondition *> _dir;
    std::vector<PointLoadCondition *> _pl;
    std::vector<std::pair<int, BoundaryConditionBase *>> _side, _vol;

private:
    const ElementPropertyCardBase *_prop = nullptr;
};

class StructuralDiscipline : public PhysicsDisciplineBase {};
class HeatConductionDiscipline : public PhysicsDisciplineBase {};

// the system's dofs: dpn variables per node of the mesh
class NonlinearSystem;
class SystemInitialization {
public:
    SystemInitialization(NonlinearSystem &sys, const Mesh &m, int dpn) : _sys(&sys), _mesh(&m), _dpn(dpn) {}
    NonlinearSystem &system() const { return *_sys; }
    const Mesh &mesh() const { return *_mesh; }
    int n_vars() const { return _dpn; }

private:
    NonlinearSystem *_sys;
    const Mesh *_mesh;
    int _dpn;
};

// translational displacements ux, uy, uz (the 3D element's rotational dofs are
// decoupled, structural_system_initialization.cpp:29-42, solid_element_3d.cpp:415-417)
class StructuralSystemInitialization : public SystemInitialization {
public:
    StructuralSystemInitialization(NonlinearSystem &sys, const Mesh &m)
        : SystemInitialization(sys, m, m.type == HEX8 ? 3 : 2) {}
};

class HeatConductionSystemInitialization : public SystemInitialization {
public:
    HeatConductionSystemInitialization(NonlinearSystem &sys, const Mesh &m) : SystemInitialization(sys, m, 1) {}
};

class NonlinearImplicitAssembly;

// one element of the mesh (stands in for MAST::GeomElem over a libMesh::Elem)
class GeomElem {
public:
    // the element with index `elem` of the system's mesh (GeomElem::init(elem, system),
    // geom_elem.cpp:133-160)
    void init(int64_t elem, const SystemInitialization &) { _id = elem; }
    int64_t id() const { return _id; }

private:
    int64_t _id = -1;
};

// Element operations of an assembly (MAST::AssemblyElemOperations,
// src/base/assembly_elem_operation.h:40-176).  The per-element calls forward to
// mg_element_calculations / mg_element_sensitivity on the assembly's problem, one
// element at a time, as MAST's own assembly loop calls them.
class AssemblyElemOperations {
public:
    virtual ~AssemblyElemOperations() {}
    // mg_physics of the element kernels for this mesh
    virtual int physics(const Mesh &m) const = 0;
    virtual void set_assembly(NonlinearImplicitAssembly &assembly) { _assembly = &assembly; }
    virtual NonlinearImplicitAssembly &get_assembly() {
        if (!_assembly) throw std::runtime_error("element operations: no assembly set");
        return *_assembly;
    }
    virtual void clear_assembly() { _assembly = nullptr; }
    virtual void set_elem_data(unsigned int, int64_t, GeomElem &) const {}
    // MAST builds the physics element here (assembly_elem_operation.cpp:195-202)
    virtual void init(const GeomElem &elem) {
        if (_elem >= 0) throw std::runtime_error("init: the previous element was not cleared");
        _elem = elem.id();
    }
    virtual void clear_elem() {
        _elem = -1;
        _sol.clear();
    }
    virtual void set_elem_solution(const RealVectorX &sol) { _sol = sol; }

protected:
    mg_problem *_problem();
    int64_t _elem = -1;
    RealVectorX _sol;
    NonlinearImplicitAssembly *_assembly = nullptr;
};

// MAST::NonlinearImplicitAssemblyElemOperations
// (src/base/nonlinear_implicit_assembly_elem_operations.h:50-105)
class NonlinearImplicitAssemblyElemOperations : public AssemblyElemOperations {
public:
    // element residual f_int - f_ext of the element's own loads and, if if_jac, its
    // Jacobian, at the solution of set_elem_solution (var-blocked element dofs)
    virtual void elem_calculations(bool if_jac, RealVectorX &vec, RealMatrixX &mat) {
        const int nd = _ndofs();
        vec.assign(nd, 0.0);
        std::vector<Real> K(if_jac ? (size_t)nd * nd : 0);
        check(mg_element_calculations(_problem(), _elem, _sol.data(), if_jac ? K.data() : nullptr, vec.data()),
              "elem_calculations");
        if (if_jac) {
            mat = RealMatrixX::Zero(nd, nd);
            for (int i = 0; i < nd; i++)
                for (int j = 0; j < nd; j++) mat(i, j) = K[(size_t)i * nd + j];
        }
    }
    // d(element residual)/dp for a parameter function ("rho_<e>", "s_<e>", "k0")
    virtual void elem_sensitivity_calculations(const FunctionBase &f, RealVectorX &vec);

protected:
    int _ndofs();
};

class StructuralNonlinearAssemblyElemOperations : public NonlinearImplicitAssemblyElemOperations {
public:
    int physics(const Mesh &m) const override {
        return m.type == HEX8 ? MG_PHYSICS_ELASTICITY_HEX8 : MG_PHYSICS_MEMBRANE_QUAD4;
    }
};

class HeatConductionNonlinearAssemblyElemOperations : public NonlinearImplicitAssemblyElemOperations {
public:
    int physics(const Mesh &) const override { return MG_PHYSICS_HEAT_QUAD4; }
};

// ------------------------------------------------------------------ outputs
class OutputAssemblyElemOperations {
public:
    virtual ~OutputAssemblyElemOperations() {}
    Real output_total() const { return _q; }
    // the derivative left by calculate_output_direct_sensitivity for parameter p
    Real output_sensitivity_total(const FunctionBase &p) const {
        auto it = _dq_dp.find(p.name());
        if (it == _dq_dp.end()) throw std::runtime_error("no sensitivity for " + p.name());
        return it->second;
    }
    Real _q = 0;
    std::map<std::string, Real> _dq_dp;
};

// compliance f.u (the configs' loads are nodal point loads, which MAST's
// ComplianceOutput does not integrate: compliance_output.cpp:71-102)
class ComplianceOutput : public OutputAssemblyElemOperations {};

// mean temperature (1/|Omega|) int T
class AverageTemperatureOutput : public OutputAssemblyElemOperations {};

// KS-aggregated von Mises stress over every element (MAST::KSStressStrainOutput,
// ks_stress_output.cpp:41-99; set_aggregation_coefficients as stress_output_base.h:246-252)
class KSStressStrainOutput : public OutputAssemblyElemOperations {
public:
    void set_aggregation_coefficients(Real p1, Real p2, Real rho, Real sigma0) {
        _p = p1;
        _p2 = p2;  // the p-norm weight and rho of the other aggregates: unused by KS
        _rho = rho;
        _sigma0 = sigma0;
    }
    void set_participating_elements_to_all() {}
    // SIMP exponent of the modulus the stress is evaluated with: the penalty example_6 sets
    // on its ElasticityFunction before evaluating the output (example_6.cpp:579-592);
    // <= 0 uses the solve's exponent
    void set_stress_penalty(Real penalty) { _penal = penalty; }
    Real get_maximum_von_mises_stress() const { return _vmax; }
    Real get_p_stress_val() const { return _p; }
    Real _p = 0, _p2 = 0, _rho = 0, _sigma0 = 0, _penal = 0, _vmax = 0;
};

// ------------------------------------------------------------------ assembly + solve
class NonlinearSystem {
public:
    NonlinearSystem() { mg_default_solve_opts(&opts); }
    Vector solution;
    mg_solve_opts opts;
    mg_solve_report last_report{};
    // Newton + Krylov on the assembly's problem; the solution is left in `solution`
    void solve(AssemblyElemOperations &elem_ops, NonlinearImplicitAssembly &assembly);
    // adjoint K^T lambda = -dq/dX for the output (compliance: lambda = -u)
    void adjoint_solve(const Vector &X, bool if_assemble_jacobian, AssemblyElemOperations &elem_ops,
                       OutputAssemblyElemOperations &output, NonlinearImplicitAssembly &assembly,
                       Vector &adjoint);
    // forward sensitivity J(X) dX/dp = -dR/dp (nonlinear_system.cpp:741-794); the result
    // is left in get_sensitivity_solution() (add_sensitivity_solution in MAST)
    void sensitivity_solve(const Vector &X, bool if_localize_sol, AssemblyElemOperations &elem_ops,
                           NonlinearImplicitAssembly &assembly, const FunctionBase &p,
                           bool if_assemble_jacobian = true);
    Vector &get_sensitivity_solution() { return _sens_sol; }

private:
    Vector _sens_sol;
};

class NonlinearImplicitAssembly {
public:
    NonlinearImplicitAssembly() {}
    ~NonlinearImplicitAssembly() { clear_discipline_and_system(); }
    NonlinearImplicitAssembly(const NonlinearImplicitAssembly &) = delete;
    NonlinearImplicitAssembly &operator=(const NonlinearImplicitAssembly &) = delete;

    void set_discipline_and_system(PhysicsDisciplineBase &discipline, SystemInitialization &system,
                                   AssemblyElemOperations &elem_ops) {
        clear_discipline_and_system();
        _disc = &discipline;
        _sys = &system;
        _ops = &elem_ops;
        elem_ops.set_assembly(*this);
    }
    void clear_discipline_and_system() {
        if (_ops) _ops->clear_assembly();
        if (_p) mg_problem_destroy(_p);
        _p = nullptr;
        _disc = nullptr;
        _sys = nullptr;
        _ops = nullptr;
    }
    // element densities of the SIMP modulus E(rho) = E0 (rmin + (1 - rmin) rho^p)
    // with E0 from the material card's "E" and Emin/penal given here
    void set_simp(const std::vector<Real> &rho, Real Emin, Real penal) {
        _rho = rho;
        _Emin = Emin;
        _penal = penal;
        _nodal = false;
        if (_p) check(mg_set_design(_p, _rho.data()), "set_simp");
    }
    // a nodal density field (example_6.cpp:104-137: the ElasticityFunction reads a
    // FIRST-order LAGRANGE "rho" through MeshFieldFunction): the modulus at each Gauss
    // point from the trilinear field; density parameters then index nodes
    void set_simp_nodal(const std::vector<Real> &rho_nodes, Real Emin, Real penal) {
        _rho = rho_nodes;
        _Emin = Emin;
        _penal = penal;
        _nodal = true;
        if (_p) check(mg_set_design_nodal(_p, _rho.data()), "set_simp_nodal");
    }
    // per-element conductivity scale s_e (heat)
    void set_conductivity_scale(const std::vector<Real> &s) {
        _scale = s;
        if (_p) check(mg_set_elem_scale(_p, _scale.data()), "set_conductivity_scale");
    }

    mg_problem *problem() {
        if (!_p) _create();
        return _p;
    }
    // mg_physics of the handle (the section's strain type decides the 3D solid branch)
    int physics() {
        problem();
        return _phys;
    }
    // the external load vector F (point loads; zero on constrained dofs)
    Vector load_vector() {
        const int64_t n = (int64_t)_sys->n_vars() * _sys->mesh().n_nodes();
        problem();
        Vector F(n);
        for (size_t i = 0; i < _ldofs.size(); i++) F(_ldofs[i]) += _lvals[i];
        for (int64_t d : _fixed) F(d) = 0.0;
        return F;
    }

    // R = f_int - f_ext at X (R, J nullable); J is the assembled CSR with
    // Dirichlet rows eliminated
    void residual_and_jacobian(const Vector &X, Vector *R, SparseMatrix *J, NonlinearSystem &) {
        mg_problem *p = problem();
        if (R) R->resize(X.size());
        check(mg_residual_and_jacobian(p, X.data(), R ? R->data() : nullptr, J != nullptr), "residual_and_jacobian");
        if (J) {
            int64_t n = 0, nnz = 0;
            int32_t nc = 0;
            check(mg_problem_info(p, &n, &nnz, &nc), "mg_problem_info");
            J->n = n;
            J->rowptr.resize(n + 1);
            J->cols.resize(nnz);
            J->vals.resize(nnz);
            check(mg_get_csr(p, J->rowptr.data(), J->cols.data(), J->vals.data()), "mg_get_csr");
        }
        _res_l2 = R ? R->l2_norm() : 0.0;
    }
    Real res_l2_norm() const { return _res_l2; }

    // dR/dp at X for one parameter: the density of element `index` (structural)
    // or k0 / the conductivity scale of element `index` (heat)
    bool sensitivity_assemble(const Vector &X, bool if_localize_sol, const FunctionBase &f, Vector &rhs,
                              bool close_vector = true) {
        (void)if_localize_sol;
        int kind;
        int64_t index;
        param_of(f, kind, index);
        rhs.resize(X.size());
        check(mg_sensitivity_assemble(problem(), X.data(), kind, index, rhs.data()), "sensitivity_assemble");
        if (close_vector) rhs.close();
        return true;
    }

    void calculate_output(const Vector &X, bool if_localize_sol, OutputAssemblyElemOperations &output) {
        (void)if_localize_sol;
        Real q = 0;
        if (dynamic_cast<ComplianceOutput *>(&output))
            check(mg_compliance(problem(), X.data(), &q, nullptr), "calculate_output");
        else if (dynamic_cast<AverageTemperatureOutput *>(&output)) {
            mg_solve_opts o;
            mg_default_solve_opts(&o);
            check(mg_mean_temperature(problem(), X.data(), &o, &q, nullptr, nullptr), "calculate_output");
        } else if (auto *ks = dynamic_cast<KSStressStrainOutput *>(&output)) {
            check(mg_ks_stress(problem(), X.data(), ks->_p, ks->_sigma0, ks->_penal, &q, &ks->_vmax, nullptr),
                  "calculate_output");
        } else
            throw std::runtime_error("calculate_output: unsupported output");
        output._q = q;
    }

    // sens[i] = lambda . dR/dp_i (+ partials of the output are not included),
    // for the parameters of every element at once; with the compliance adjoint
    // lambda = -u this is dC/drho_e = -u_e^T dK_e/drho_e u_e
    void calculate_output_adjoint_sensitivity_multiple_parameters_no_direct(
        const Vector &X, bool if_localize_sol, const Vector &adj_sol,
        const std::vector<const FunctionBase *> &p_vec, AssemblyElemOperations &elem_ops,
        OutputAssemblyElemOperations &output, std::vector<Real> &sens) {
        (void)if_localize_sol;
        (void)elem_ops;
        sens.assign(p_vec.size(), 0.0);
        mg_problem *p = problem();
        if (dynamic_cast<ComplianceOutput *>(&output) && physics() != MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) {
            // the library forms -u^T dK/drho u with its own adjoint (lambda = -u)
            for (size_t i = 0; i < X.size(); i++)
                if (std::fabs(adj_sol(i) + X(i)) > 1e-12 * (1 + std::fabs(X(i))))
                    throw std::runtime_error("compliance adjoint must be -u");
            std::vector<Real> dc(_nodal ? _sys->mesh().n_nodes() : _sys->mesh().n_elem());
            Real c = 0;
            check(mg_compliance(p, X.data(), &c, dc.data()), "adjoint sensitivity");
            for (size_t i = 0; i < p_vec.size(); i++) {
                int kind;
                int64_t index;
                param_of(*p_vec[i], kind, index);
                sens[i] = dc[index];
            }
            return;
        }
        // general outputs: lambda . dR/dp_i, one assembled dR/dp per parameter
        Vector d;
        for (size_t i = 0; i < p_vec.size(); i++) {
            sensitivity_assemble(X, false, *p_vec[i], d);
            Real s = 0;
            for (size_t k = 0; k < X.size(); k++) s += adj_sol(k) * d(k);
            sens[i] = s;
        }
    }

    // the total design derivative of a KS stress output in one call: what MAST forms as
    // adjoint_solve + calculate_output_adjoint_sensitivity_multiple_parameters_no_direct (the
    // adjoint term, at the solve's exponent) + calculate_output_direct_sensitivity (the term
    // through the stress modulus), example_6.cpp:798-874; density parameters only
    void calculate_output_total_sensitivity(const Vector &X, KSStressStrainOutput &output,
                                            const std::vector<const FunctionBase *> &p_vec,
                                            std::vector<Real> &sens) {
        std::vector<Real> d(_sys->mesh().n_elem());
        Real q = 0;
        check(mg_ks_stress(problem(), X.data(), output._p, output._sigma0, output._penal, &q, &output._vmax,
                           d.data()),
              "KS stress sensitivity");
        output._q = q;
        sens.assign(p_vec.size(), 0.0);
        for (size_t i = 0; i < p_vec.size(); i++) {
            int kind;
            int64_t index;
            param_of(*p_vec[i], kind, index);
            if (kind != MG_PARAM_DENSITY) throw std::runtime_error("KS stress sensitivity: density parameters only");
            sens[i] = d[index];
        }
    }

    // dq/dX of the output at X, zero on constrained dofs (assembly_base.cpp:336-429)
    void calculate_output_derivative(const Vector &X, bool if_localize_sol, OutputAssemblyElemOperations &output,
                                     Vector &dq_dX) {
        (void)if_localize_sol;
        int kind;
        if (dynamic_cast<ComplianceOutput *>(&output)) kind = MG_OUTPUT_COMPLIANCE;
        else if (dynamic_cast<AverageTemperatureOutput *>(&output)) kind = MG_OUTPUT_MEAN_TEMPERATURE;
        else throw std::runtime_error("calculate_output_derivative: unsupported output");
        dq_dX.resize(X.size());
        check(mg_output_derivative(problem(), kind, X.data(), dq_dX.data()), "calculate_output_derivative");
    }

    // dq/dp = partial dq/dp + dq/dX . dX/dp (assembly_base.cpp:434-520): with dXdp from
    // NonlinearSystem::sensitivity_solve this is the total (direct) sensitivity, without
    // it the partial derivative.  The compliance F.X and the mean temperature do not
    // depend on the density, k0 or the conductivity scale explicitly, so their partial
    // derivatives are zero.  The value is left in output.output_sensitivity_total(p).
    void calculate_output_direct_sensitivity(const Vector &X, bool if_localize_sol, const Vector *dXdp,
                                             bool if_localize_sol_sens, const FunctionBase &p,
                                             OutputAssemblyElemOperations &output) {
        (void)if_localize_sol_sens;
        Real s = 0.0;
        if (dXdp) {
            Vector dq;
            calculate_output_derivative(X, if_localize_sol, output, dq);
            for (size_t i = 0; i < X.size(); i++) s += dq(i) * (*dXdp)(i);
        } else if (!dynamic_cast<ComplianceOutput *>(&output) && !dynamic_cast<AverageTemperatureOutput *>(&output))
            throw std::runtime_error("calculate_output_direct_sensitivity: unsupported output");
        output._dq_dp[p.name()] = s;
    }

    // element-parameter functions: "rho_<e>" / "s_<e>" name element e's density
    // or conductivity scale; "k0" the base conductivity
    static std::string elem_param_name(const char *kind, int64_t e) { return std::string(kind) + "_" + std::to_string(e); }

    // the (mg_sensitivity_assemble kind, index) a parameter function names
    static void param_of(const FunctionBase &f, int &kind, int64_t &index) {
        const std::string &nm = f.name();
        if (nm == "k0") { kind = MG_PARAM_K0; index = 0; return; }
        const size_t u = nm.find('_');
        if (u == std::string::npos) throw std::runtime_error("unknown parameter " + nm);
        const std::string k = nm.substr(0, u);
        index = std::stoll(nm.substr(u + 1));
        if (k == "rho") kind = MG_PARAM_DENSITY;
        else if (k == "s") kind = MG_PARAM_ELEM_SCALE;
        else throw std::runtime_error("unknown parameter " + nm);
    }

    void _create() {
        if (!_disc || !_sys || !_ops) throw std::runtime_error("assembly has no discipline and system");
        const Mesh &m = _sys->mesh();
        const int dpn = _sys->n_vars();
        const ElementPropertyCardBase &prop = _disc->property();
        const IsotropicMaterialPropertyCard &mat = prop.get_material();
        mg_material_desc md{};
        int phys = _ops->physics(m);
        if (phys == MG_PHYSICS_ELASTICITY_HEX8 && prop.strain_type() == NONLINEAR_STRAIN)
            phys = MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR;
        _phys = phys;
        if (phys == MG_PHYSICS_HEAT_QUAD4) {
            md.k0 = mat.value("k_th");
            md.k_beta = mat.contains("k_beta") ? mat.value("k_beta") : 0.0;
            md.thickness = prop.contains("h") ? prop.value("h") : 1.0;
            md.E0 = 1.0;
            md.penal = 1.0;
        } else {
            md.E0 = mat.value("E");
            md.nu = mat.value("nu");
            md.Emin = _Emin;
            md.penal = _penal;
            md.thickness = prop.contains("h") ? prop.value("h") : 1.0;
        }
        // Dirichlet dofs and point loads
        std::set<int64_t> fixed;
        for (auto *bc : _disc->_dir)
            for (int64_t n : m.boundary_nodes(bc->boundary_id()))
                for (unsigned v : bc->vars())
                    if ((int)v < dpn) fixed.insert(dpn * n + v);
        _fixed.assign(fixed.begin(), fixed.end());
        _ldofs.clear();
        _lvals.clear();
        for (auto *pl : _disc->_pl)
            for (int64_t n : pl->get_nodes())
                for (int v = 0; v < dpn && v < (int)pl->load().size(); v++)
                    if (pl->load()[v] != 0.0) {
                        _ldofs.push_back(dpn * n + v);
                        _lvals.push_back(pl->load()[v]);
                    }
        mg_bc_desc bc{};
        bc.n_fixed = (int64_t)_fixed.size();
        bc.fixed_dofs = _fixed.data();
        bc.n_point_loads = (int64_t)_ldofs.size();
        bc.load_dofs = _ldofs.data();
        bc.load_values = _lvals.data();
        _ce.clear();
        _cs.clear();
        for (auto &sl : _disc->_side)
            if (sl.second->type() == CONVECTION_HEAT_FLUX)
                for (auto &es : m.boundary_sides(sl.first)) {
                    _ce.push_back(es.first);
                    _cs.push_back(es.second);
                    bc.conv_h = sl.second->value("convection_coeff");
                    bc.conv_Tinf = sl.second->value("ambient_temperature");
                }
        bc.n_conv = (int64_t)_ce.size();
        bc.conv_elems = _ce.data();
        bc.conv_sides = _cs.data();
        if (!_disc->_vol.empty()) {
            // volume heat source on the elements listed by the subdomain id:
            // subdomain -1 = every element; otherwise the caller's q field
            _src.assign(m.n_elem(), 0.0);
            for (auto &vl : _disc->_vol)
                if (vl.second->type() == HEAT_SOURCE) {
                    const Real q = vl.second->value("heat_source");
                    for (int64_t e = 0; e < m.n_elem(); e++)
                        if (vl.first < 0 || (e < (int64_t)_subdomain.size() && _subdomain[e] == vl.first))
                            _src[e] += q;
                }
            bc.source_elem = _src.data();
        }
        mg_mesh_desc mesh{};
        mesh.physics = phys;
        mesh.n_nodes = m.n_nodes();
        mesh.n_elems = m.n_elem();
        mesh.coords = m.coords.data();
        mesh.conn = m.conn.data();
        mesh.grid_nx = m.nx;
        mesh.grid_ny = m.ny;
        mesh.grid_nz = m.nz;
        check(mg_problem_create(&mesh, &md, &bc, &_p), "mg_problem_create");
        // surface pressure (3D solid faces) and heat flux (2D edges) side loads
        std::vector<int32_t> se, ss;
        std::vector<Real> sv;
        for (auto &sl : _disc->_side) {
            const BoundaryConditionType t = sl.second->type();
            if (t != SURFACE_PRESSURE && t != HEAT_FLUX) continue;
            const Real v = sl.second->value(t == SURFACE_PRESSURE ? "pressure" : "heat_flux");
            for (auto &es : m.boundary_sides(sl.first)) {
                se.push_back(es.first);
                ss.push_back(es.second);
                sv.push_back(v);
            }
        }
        if (!se.empty())
            check(mg_set_side_loads(_p, (int64_t)se.size(), se.data(), ss.data(), sv.data()), "side loads");
        if (!_rho.empty())
            check(_nodal ? mg_set_design_nodal(_p, _rho.data()) : mg_set_design(_p, _rho.data()), "set_simp");
        if (!_scale.empty()) check(mg_set_elem_scale(_p, _scale.data()), "set_conductivity_scale");
    }

public:
    // subdomain id per element (volume loads on subdomains); empty = none
    std::vector<int> _subdomain;

private:
    PhysicsDisciplineBase *_disc = nullptr;
    SystemInitialization *_sys = nullptr;
    AssemblyElemOperations *_ops = nullptr;
    mg_problem *_p = nullptr;
    std::vector<Real> _rho, _scale, _lvals, _src;
    bool _nodal = false;  // _rho per node (set_simp_nodal) rather than per element
    std::vector<int64_t> _fixed, _ldofs;
    std::vector<int32_t> _ce, _cs;
    Real _Emin = 1e-9, _penal = 3.0, _res_l2 = 0.0;
    int _phys = -1;
};

inline mg_problem *AssemblyElemOperations::_problem() {
    if (_elem < 0) throw std::runtime_error("element operations: init(elem) was not called");
    return get_assembly().problem();
}

inline int NonlinearImplicitAssemblyElemOperations::_ndofs() {
    mg_problem *p = _problem();
    int64_t n = 0, nnz = 0;
    int32_t nc = 0;
    check(mg_problem_info(p, &n, &nnz, &nc), "mg_problem_info");
    const int phys = get_assembly().physics();
    const int nd = (phys == MG_PHYSICS_HEAT_QUAD4) ? 4 : (phys == MG_PHYSICS_MEMBRANE_QUAD4) ? 8 : 24;
    if ((int)_sol.size() != nd) throw std::runtime_error("set_elem_solution: wrong element vector size");
    return nd;
}

inline void NonlinearImplicitAssemblyElemOperations::elem_sensitivity_calculations(const FunctionBase &f,
                                                                                  RealVectorX &vec) {
    const int nd = _ndofs();
    int kind;
    int64_t index;
    NonlinearImplicitAssembly::param_of(f, kind, index);
    vec.assign(nd, 0.0);
    check(mg_element_sensitivity(_problem(), _elem, _sol.data(), kind, index, vec.data()),
          "elem_sensitivity_calculations");
}

inline void NonlinearSystem::sensitivity_solve(const Vector &X, bool, AssemblyElemOperations &,
                                               NonlinearImplicitAssembly &assembly, const FunctionBase &p,
                                               bool) {
    int kind;
    int64_t index;
    NonlinearImplicitAssembly::param_of(p, kind, index);
    _sens_sol.resize(X.size());
    check(mg_sensitivity_solve(assembly.problem(), X.data(), kind, index, &opts, _sens_sol.data()),
          "NonlinearSystem::sensitivity_solve");
}

inline void NonlinearSystem::solve(AssemblyElemOperations &, NonlinearImplicitAssembly &assembly) {
    mg_problem *p = assembly.problem();
    int64_t n = 0, nnz = 0;
    int32_t nc = 0;
    check(mg_problem_info(p, &n, &nnz, &nc), "mg_problem_info");
    if ((int64_t)solution.size() != n) solution.resize(n);
    check(mg_solve(p, &opts, solution.data(), &last_report), "NonlinearSystem::solve");
}

inline void NonlinearSystem::adjoint_solve(const Vector &X, bool, AssemblyElemOperations &,
                                           OutputAssemblyElemOperations &output,
                                           NonlinearImplicitAssembly &assembly, Vector &adjoint) {
    if (dynamic_cast<KSStressStrainOutput *>(&output))
        throw std::runtime_error("adjoint_solve: the GPU path forms the KS stress adjoint inside mg_ks_stress; "
                                 "use NonlinearImplicitAssembly::calculate_output_total_sensitivity");
    if (!dynamic_cast<ComplianceOutput *>(&output))
        throw std::runtime_error("adjoint_solve: the GPU path forms the mean-temperature adjoint inside "
                                 "mg_mean_temperature; use calculate_output_adjoint_sensitivity");
    if (assembly.physics() == MG_PHYSICS_ELASTICITY_HEX8_NONLINEAR) {
        // C = F.u: K_T(u)^T lambda = -dC/du = -F on the tangent at X
        Vector rhs = assembly.load_vector();
        for (size_t i = 0; i < rhs.size(); i++) rhs(i) = -rhs(i);
        adjoint.resize(X.size());
        check(mg_adjoint_solve(assembly.problem(), X.data(), rhs.data(), &opts, adjoint.data()),
              "NonlinearSystem::adjoint_solve");
        return;
    }
    // compliance is self-adjoint: K lambda = -f  =>  lambda = -u (example_6.cpp:877-939)
    adjoint.resize(X.size());
    for (size_t i = 0; i < X.size(); i++) adjoint(i) = -X(i);
}

}  // namespace MAST
