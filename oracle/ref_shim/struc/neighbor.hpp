// Stand-in for the reference's struc/neighbor.hpp, which nnp/nnp.hpp includes but the reference's
// sources do not contain. It provides what nnp/nnp.cpp reads from a NeighborList
// (nnp.cpp:343-348, 478-500): per centre atom i, size(i) entries, each with the neighbour's type
// index, its atom index, whether it receives the Newton's-third-law reaction (min), the pair
// vector r = x_i - x_j (image included) and its length dr. The caller fills the rows from an
// existing list. Test infrastructure for pinning the oracle.
#pragma once
#include <vector>
#include <Eigen/Dense>

class NeighborEntry {
public:
    int type_ = 0, index_ = 0;
    bool min_ = true;
    Eigen::Vector3d r_;
    double dr_ = 0;
    int type() const { return type_; }
    int index() const { return index_; }
    bool min() const { return min_; }
    const Eigen::Vector3d& r() const { return r_; }
    double dr() const { return dr_; }
};

class NeighborList {
    std::vector<std::vector<NeighborEntry>> rows_;

public:
    void resize(int natoms) { rows_.assign(natoms, std::vector<NeighborEntry>()); }
    void add(int i, const NeighborEntry& e) { rows_[i].push_back(e); }
    int size(int i) const { return (int)rows_[i].size(); }
    const NeighborEntry& neigh(int i, int j) const { return rows_[i][j]; }
};
