// Host-side container of a built plan (DevPot plus the parameter arrays before upload).
#pragma once
#include <vector>
#include "plan.hpp"
#include "potential.hpp"

namespace ann {

struct PlanHost {
    DevPot pot;
    int slots = 8;                       // fast-path slots per angular block (fastNG * 8)
    std::vector<double> rs, reta, aeta, zeta, alam;
    std::vector<int> agrp, slot2ref;
    std::vector<double> w, wt, b, inpw, inpb;
};

void build_plan(const Potential& p, PlanHost& out);

}  // namespace ann
