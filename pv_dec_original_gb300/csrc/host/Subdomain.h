// SubDomain with the reference's constructor SubDomain(Geometry&)
// (Subdomain.h:66).  The reference builds one heap Node per point, links
// neighbours with shared_ptr and splits the domain over MPI ranks
// (Subdomain.cpp:3-32); here the whole lattice is one device-resident
// domain, built by lbm_set_geometry when a Simulation starts.  SubDomain
// carries the lattice and the solver options.
#pragma once
#include <memory>

#include "ComplexGeometry.h"
#include "LatticeModel.h"

struct LbmOptions {
    int Q = 19;                  // LBM_D3Q19 / LBM_D3Q27
    int precision = LBM_F64;     // FP64 reproduces the reference bit for bit (parity mode)
    int mode = LBM_PARITY;       // LBM_PARITY (reference semantics) or LBM_PHYSICS
    int device = 0;
};

class SubDomain {
public:
    Geometry Geometry_;
    std::shared_ptr<VelocitySet> m_velSet;
    LbmOptions options;
    int my_Nx = 0, my_Ny = 0, my_Nz = 0;

    SubDomain() = default;
    explicit SubDomain(Geometry& geometry, LbmOptions opt = LbmOptions());
    const std::shared_ptr<VelocitySet> GetVelSet() { return m_velSet; }
};
