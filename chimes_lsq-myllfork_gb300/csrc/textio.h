// Text files of the fit and the coefficient reader of params.txt.
#pragma once
#include <string>
#include <vector>

#include "model.h"
#include "session.h"

namespace cg {

// A.txt, b.txt, b-labeled.txt, natoms.txt and dim.txt of a frame batch in dir
// (A_MAT::PRINT_FRAME / CLEANUP_FILES, src/A_Matrix.C:210-720): A host, row-major.
void write_lsq_files(const Model& m, const FrameBatch& fb, const double* A, int64_t lda, const std::string& dir,
                     bool with_constraints = true);

// Coefficient vector (A-column order) of a params.txt text for this model.
std::vector<double> params_txt_coefficients(const Model& m, const std::string& text);

}  // namespace cg
