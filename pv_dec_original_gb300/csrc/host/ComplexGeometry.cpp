#include "ComplexGeometry.h"

#include <cmath>
#include <stdexcept>

Geometry::Geometry(const std::string& FileName, std::shared_ptr<VelocitySet> velSet, double s, char rd)
    : stlFileName(FileName), spacing(s), raydirection(rd), m_velSet(std::move(velSet)) {
    globalTriangles = Reader_.readSTLASCII(stlFileName);
    GetSubBoundingBox();
    labelPoints();
}

Geometry::Geometry(const std::vector<Triangle>& tris, std::shared_ptr<VelocitySet> velSet, double s,
                   const BoundingBox& rayBox, const double org[3], const int dims[3])
    : globalTriangles(tris), spacing(s), m_velSet(std::move(velSet)), rayBox_(rayBox), referenceBox_(false) {
    boundingbox = rayBox;
    origin[0] = org[0]; origin[1] = org[1]; origin[2] = org[2];
    nx = dims[0]; ny = dims[1]; nz = dims[2];
    labelPoints();
}

void Geometry::GetSubBoundingBox() {
    if (globalTriangles.empty()) throw std::runtime_error("Geometry: no triangles read from " + stlFileName);
    std::vector<double> rows = triangles_to_rows(globalTriangles);
    lbm_vox_desc d{};
    d.spacing = spacing;
    d.reference_bbox = 1;
    if (lbm_voxelize(rows.data(), (int64_t)globalTriangles.size(), &d, nullptr) != LBM_OK)
        throw std::runtime_error(std::string("Geometry: ") + lbm_last_global_error());
    boundingbox = BoundingBox{d.bbox[0], d.bbox[1], d.bbox[2], d.bbox[3], d.bbox[4], d.bbox[5]};
    origin[0] = d.origin[0]; origin[1] = d.origin[1]; origin[2] = d.origin[2];
    nx = d.dims[0]; ny = d.dims[1]; nz = d.dims[2];
    rayBox_ = boundingbox;
    referenceBox_ = true;
}

void Geometry::labelPoints() {
    std::vector<double> rows = triangles_to_rows(globalTriangles);
    lbm_vox_desc d{};
    d.spacing = spacing;
    d.reference_bbox = 0;
    const double bb[6] = {rayBox_.min_x, rayBox_.max_x, rayBox_.min_y, rayBox_.max_y, rayBox_.min_z, rayBox_.max_z};
    for (int q = 0; q < 6; ++q) d.bbox[q] = bb[q];
    for (int q = 0; q < 3; ++q) d.origin[q] = origin[q];
    d.dims[0] = nx; d.dims[1] = ny; d.dims[2] = nz;
    mask.assign((size_t)nx * ny * nz, 0);
    if (lbm_voxelize(rows.data(), (int64_t)globalTriangles.size(), &d, mask.data()) != LBM_OK)
        throw std::runtime_error(std::string("Geometry::labelPoints: ") + lbm_last_global_error());
    fluidCount = d.fluid_count;
    rayTests = d.ray_tests;
}

std::vector<Point> Geometry::findBoundaryPoints() const {
    std::vector<Point> out;
    const int Q = m_velSet ? m_velSet->Get_nDirections() : 19;
    LatticeModel lm(Q);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                if (!IsFluid(i, j, k)) continue;
                bool b = false;
                for (int q = 0; q < Q && !b; ++q) {
                    std::vector<int> c = lm.GetDirection(q);
                    b = !IsFluid(i + c[0], j + c[1], k + c[2]);
                }
                if (b) out.push_back(PointAt(i, j, k));
            }
    return out;
}

void Geometry::AddInlet(int face, int plane, double scale) {
    lbm_bc_spec r{};
    r.kind = LBM_BC_VELOCITY; r.face = face; r.plane = plane; r.value = scale;
    boundaryRules.push_back(r);
}

void Geometry::AddParabolicInlet(int face, int plane, double c1, double c2, double R, double scale) {
    lbm_bc_spec r{};
    r.kind = LBM_BC_VELOCITY; r.face = face; r.plane = plane; r.value = scale;
    r.profile = 1; r.c1 = c1; r.c2 = c2; r.R = R;
    boundaryRules.push_back(r);
}

void Geometry::AddPressureOutlet(int face, int plane, double density) {
    lbm_bc_spec r{};
    r.kind = LBM_BC_PRESSURE; r.face = face; r.plane = plane; r.value = density;
    boundaryRules.push_back(r);
}

void Geometry::UsePVPreset() {
    // ComplexGeometry.cpp:1378-1408: |coordinate - c| <= 0.01 on the plane
    // axis and open intervals on the two others (x < y < z order)
    struct R { int kind, face; double c, lo1, hi1, lo2, hi2; };
    const R rules[4] = {
        {LBM_BC_REF_INLET, LBM_FACE_XMIN, -16.9538, -191.0, -187.0, -118.0, -114.0},
        {LBM_BC_REF_OUTLET_YMAX, LBM_FACE_YMAX, -170.016, 2.0, 5.0, -109.0, -106.0},
        {LBM_BC_REF_OUTLET_ZMIN, LBM_FACE_ZMIN, -110.0, -27.0, -25.0, -198.0, -195.0},
        {LBM_BC_REF_OUTLET_ZMIN, LBM_FACE_ZMIN, -123.0, -33.0, -30.0, -189.0, -186.0},
    };
    boundaryRules.clear();
    for (const R& x : rules) {
        lbm_bc_spec r{};
        r.kind = x.kind; r.face = x.face; r.plane = -1; r.value = 1.0;
        r.region = 1; r.coord = x.c; r.tol = 1e-2;
        r.lo[0] = x.lo1; r.hi[0] = x.hi1; r.lo[1] = x.lo2; r.hi[1] = x.hi2;
        boundaryRules.push_back(r);
    }
}
