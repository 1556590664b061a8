// Lattice tables with the reference's accessors (VelocitySet.h:15-24,
// LatticeModel.h:9-13): weights, directions, c_s^2, opposite direction and
// the unknown-population sets per face normal (LatticeModel.cpp:96-101).
// D3Q19 keeps the reference's numbering (rest population last), D3Q27 the
// reference's D3Q27 numbering (rest population first).
#pragma once
#include <utility>
#include <vector>

class VelocitySet {
public:
    VelocitySet(int Q);
    virtual ~VelocitySet() = default;
    double GetWeight(int dir) const;
    std::vector<int> GetDirection(int dir) const;
    double Get_c_square(int dir) const;
    int Get_nDimensions() const { return 3; }
    int Get_nDirections() const { return Q_; }
    virtual int OppositeDirection(int dir) const;
    // (unknown directions, outward face normal) per face, as m_UnkDisNor
    std::vector<std::pair<std::vector<int>, std::vector<double>>> m_UnkDisNor;

protected:
    int Q_;
};

class LatticeModel : public VelocitySet {
public:
    explicit LatticeModel(int Q = 19);
    std::vector<std::pair<std::vector<int>, std::vector<double>>> Pair0fNormalUnkDis() const { return m_UnkDisNor; }
};
