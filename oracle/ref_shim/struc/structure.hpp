// Stand-in for the reference's struc/structure.hpp, which nnp/nnp.cpp and nnp/nnh.cpp include but
// the reference's sources do not contain. It provides only what nnp/nnp.cpp calls on a Structure
// (NNP::init / symm / energy / force / compute, nnp.cpp:316-736): per-atom type name, type index,
// position, force and symmetry-function vector, the lattice vectors R (columns), the energy,
// and diff(a, b, r) = a - b, the difference that the verlet::List functions correct by the image
// (nnp.cpp:394-395). The caller fills it from arrays. resize(n, nall) keeps nall atoms of which
// the first n are the structure's own (nAtoms, the centres); the others are ghost atoms that only
// appear as neighbours and receive forces, as in an MD engine's domain. Test infrastructure for
// pinning the oracle.
#pragma once
#include <string>
#include <vector>
#include <Eigen/Dense>
#include "struc/structure_fwd.hpp"

class Structure {
    std::vector<std::string> name_;
    std::vector<int> type_;
    std::vector<Eigen::Vector3d> posn_, force_;
    std::vector<Eigen::VectorXd> symm_;
    Eigen::Matrix3d R_;
    double pe_ = 0;
    int n_ = 0;

public:
    void resize(int n) { resize(n, n); }
    void resize(int n, int nall) {
        n_ = n;
        name_.assign(nall, std::string());
        type_.assign(nall, 0);
        posn_.assign(nall, Eigen::Vector3d());
        force_.assign(nall, Eigen::Vector3d());
        symm_.assign(nall, Eigen::VectorXd());
    }
    int nAtoms() const { return n_; }
    std::string& name(int i) { return name_[i]; }
    const std::string& name(int i) const { return name_[i]; }
    int& type(int i) { return type_[i]; }
    const int& type(int i) const { return type_[i]; }
    Eigen::Vector3d& posn(int i) { return posn_[i]; }
    const Eigen::Vector3d& posn(int i) const { return posn_[i]; }
    Eigen::Vector3d& force(int i) { return force_[i]; }
    const Eigen::Vector3d& force(int i) const { return force_[i]; }
    Eigen::VectorXd& symm(int i) { return symm_[i]; }
    const Eigen::VectorXd& symm(int i) const { return symm_[i]; }
    Eigen::Matrix3d& R() { return R_; }
    const Eigen::Matrix3d& R() const { return R_; }
    double& pe() { return pe_; }
    const double& pe() const { return pe_; }
    void diff(const Eigen::Vector3d& a, const Eigen::Vector3d& b, Eigen::Vector3d& r) const { r = a - b; }
};
