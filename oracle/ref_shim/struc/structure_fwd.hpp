// Stand-in for the reference's struc/structure_fwd.hpp, which its sources include but do not
// contain (see structure.hpp beside this file).
#pragma once
class Structure;
