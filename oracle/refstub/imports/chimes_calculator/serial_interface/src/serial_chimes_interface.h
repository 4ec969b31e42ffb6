// Stand-in for the external chimes_calculator serial interface header.
//
// The reference includes this header from an un-vendored submodule
// (chimes_calculator, cloned by the reference's clone-all.sh).  It is used only by
// the SERIAL_CHIMES pair type, which is not on the design-matrix / Chebyshev force
// path.  Every method aborts so that reaching that pair type fails loudly.
// This file is test infrastructure: it lets oracle/build_ref.sh compile the
// reference sources into oracle/_ref/ for parity checks.
#ifndef CHIMES_GB300_REFSTUB_SERIAL_CHIMES_INTERFACE_H
#define CHIMES_GB300_REFSTUB_SERIAL_CHIMES_INTERFACE_H

#include <cstdlib>
#include <string>
#include <vector>

struct serial_chimes_interface {
    explicit serial_chimes_interface(bool) {}
    void init_chimesFF(std::string, int) { std::abort(); }
    void calculate(std::vector<double>&, std::vector<double>&, std::vector<double>&,
                   std::vector<double>&, std::vector<double>&, std::vector<double>&,
                   std::vector<std::string>&, double&, std::vector<std::vector<double>>&,
                   std::vector<double>&) { std::abort(); }
};

#endif
