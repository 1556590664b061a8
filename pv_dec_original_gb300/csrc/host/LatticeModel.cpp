#include "LatticeModel.h"

#include <stdexcept>

namespace {

const int C19[19][3] = {{1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},   {0, 0, -1}, {1, 1, 0},
                        {1, -1, 0}, {1, 0, 1},  {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0}, {-1, 0, 1}, {-1, 0, -1},
                        {0, 1, 1},  {0, 1, -1}, {0, -1, 1}, {0, -1, -1}, {0, 0, 0}};
const int C27[27][3] = {{0, 0, 0},   {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                        {1, 1, 0},   {1, -1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},
                        {-1, 0, -1}, {0, 1, 1},  {0, 1, -1}, {0, -1, 1},  {0, -1, -1}, {1, 1, 1}, {-1, -1, -1},
                        {1, 1, -1},  {-1, -1, 1}, {1, -1, 1}, {-1, 1, -1}, {1, -1, -1}, {-1, 1, 1}};

const int* dir(int Q, int q) { return Q == 19 ? C19[q] : C27[q]; }

}  // namespace

VelocitySet::VelocitySet(int Q) : Q_(Q) {
    if (Q != 19 && Q != 27) throw std::invalid_argument("VelocitySet: Q must be 19 or 27");
    // faces: +x, -x, -y, +y, +z, -z as listed in the reference (LatticeModel.cpp:96-101)
    const int normals[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (const auto& nn : normals) {
        std::vector<int> unk;
        for (int q = 0; q < Q; ++q) {
            const int* c = dir(Q, q);
            if (c[0] * nn[0] + c[1] * nn[1] + c[2] * nn[2] == 1) unk.push_back(q);
        }
        m_UnkDisNor.push_back({unk, {double(nn[0]), double(nn[1]), double(nn[2])}});
    }
}

double VelocitySet::GetWeight(int q) const {
    if (q < 0 || q >= Q_) throw std::out_of_range("direction");
    if (Q_ == 19) return q < 6 ? 2.0 / 36.0 : (q < 18 ? 1.0 / 36.0 : 12.0 / 36.0);
    return q == 0 ? 8.0 / 27.0 : (q < 7 ? 2.0 / 27.0 : (q < 19 ? 1.0 / 54.0 : 1.0 / 216.0));
}

std::vector<int> VelocitySet::GetDirection(int q) const {
    if (q < 0 || q >= Q_) throw std::out_of_range("direction");
    const int* c = dir(Q_, q);
    return {c[0], c[1], c[2]};
}

double VelocitySet::Get_c_square(int) const { return 1.0 / 3.0; }

int VelocitySet::OppositeDirection(int q) const {
    if (q < 0 || q >= Q_) throw std::out_of_range("direction");
    const int* c = dir(Q_, q);
    for (int p = 0; p < Q_; ++p) {
        const int* d = dir(Q_, p);
        if (d[0] == -c[0] && d[1] == -c[1] && d[2] == -c[2]) return p;
    }
    return q;
}

LatticeModel::LatticeModel(int Q) : VelocitySet(Q) {}
