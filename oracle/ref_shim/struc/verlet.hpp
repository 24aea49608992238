// Stand-in for the reference's struc/verlet.hpp, which nnp/nnp.hpp includes but the reference's
// sources do not contain. It provides what nnp/nnp.cpp reads from a verlet::List
// (nnp.cpp:386-395, 537-550): per centre atom i, size(i) entries, each with the neighbour's atom
// index and its image as a vector of lattice-vector multiples (cell), from which the functions
// form the pair vector x_i - x_j - R cell themselves. Test infrastructure for pinning the oracle.
#pragma once
#include <vector>
#include <Eigen/Dense>

namespace verlet {

class Entry {
public:
    int index_ = 0;
    Eigen::Vector3d cell_;
    int index() const { return index_; }
    const Eigen::Vector3d& cell() const { return cell_; }
};

class List {
    std::vector<std::vector<Entry>> rows_;

public:
    void resize(int natoms) { rows_.assign(natoms, std::vector<Entry>()); }
    void add(int i, const Entry& e) { rows_[i].push_back(e); }
    int size(int i) const { return (int)rows_[i].size(); }
    const Entry& neigh(int i, int j) const { return rows_[i][j]; }
};

}  // namespace verlet
