#include "Subdomain.h"

#include <stdexcept>

SubDomain::SubDomain(Geometry& geometry, LbmOptions opt) : Geometry_(geometry), options(opt) {
    m_velSet = geometry.m_velSet ? geometry.m_velSet : std::make_shared<LatticeModel>(opt.Q);
    if (m_velSet->Get_nDirections() != options.Q)
        throw std::invalid_argument("SubDomain: velocity set and options disagree on Q");
    my_Nx = geometry.nx;
    my_Ny = geometry.ny;
    my_Nz = geometry.nz;
}
