// Test harness: the library's potential-file parser and writer (ann_gb300/csrc/potential.cpp,
// Potential::read_text / write_text) built for the CPU by tests/test_potential_io.py, so that the
// files the library writes can be compared with the reference's own NNP::read / NNP::write
// without a GPU. Not part of the library.
#include <cstdio>
#include <cstring>
#include <string>
#include "potential.hpp"

extern "C" {

// parse `in`, write it back into out[cap]; returns 0, the size needed (negative) when cap is too
// small, or 1 with the parser's message in err[errcap]
int pio_rewrite(const char* in, char* out, int cap, char* err, int errcap) {
    try {
        ann::Potential p;
        p.read_text(in);
        const std::string s = p.write_text();
        if ((int)s.size() + 1 > cap) return -(int)(s.size() + 1);
        std::memcpy(out, s.c_str(), s.size() + 1);
        return 0;
    } catch (std::exception& e) {
        std::snprintf(err, (size_t)errcap, "%s", e.what());
        return 1;
    }
}

}  // extern "C"
