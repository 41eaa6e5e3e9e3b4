/* Host pivoting analysis of the circuit matrix; see sparse.cpp. */
#ifndef NGSF_SPARSE_H
#define NGSF_SPARSE_H

#include <string>
#include <vector>

#include "circuit.h"

namespace ngsf {

/* Factor the n x n matrix given in CSC (0-based rows) with threshold
 * Markowitz pivoting and fill the LU plan fields of img (pivot sequence,
 * L+U layout, update lists, level schedules, a_lupos).  Returns false with
 * err set when the matrix is structurally or numerically singular. */
bool plan_lu(int n, const std::vector<int> &cp, const std::vector<int> &ri,
             const std::vector<double> &ax, double pivrel, double pivtol,
             Image &img, std::string &err);

/* KLU's block triangular analysis of the pattern (btf_maxtrans +
 * btf_strongcomp): the number of diagonal blocks and the largest block's
 * size.  Returns false when the pattern is structurally singular. */
bool btf_analyze(int n, const std::vector<int> &cp, const std::vector<int> &ri, int &nblocks,
                 int &largest);

}  // namespace ngsf

#endif
