// read.hpp - FROSTT .tns reading and writing for the drop-in Tensor, as the
// reference's read.hpp:58-142 does: lines of `i1 i2 ... iN value`,
// coordinates taken as given (no 1-based shift), lines that do not start with
// a digit skipped, the first digit line skipped when has_header is true.
// The shape is the per-mode max over every data row (the reference's reader
// leaves the first row out, read.hpp:79-89; callers run _infer_shape anyway).
#ifndef FASTCC_GB300_READ_HPP
#define FASTCC_GB300_READ_HPP

#include <cctype>
#include <fstream>
#include <sstream>

#include "contract.hpp"

template <class DT> Tensor<DT>::Tensor(std::string fname, bool has_header) {
  std::ifstream file(fname);
  if (!file) throw fcc::Error(FCC_ERR_ARG, "cannot open " + fname);
  std::string line;
  int dims = 0;
  while (std::getline(file, line)) {
    if (line.empty() || !std::isdigit(static_cast<unsigned char>(line[0]))) continue;
    if (has_header) {
      has_header = false;
      continue;
    }
    std::istringstream in(line);
    std::vector<std::string> tok;
    std::string t;
    while (in >> t) tok.push_back(t);
    if (tok.size() < 2) continue;
    std::vector<int> c;
    for (size_t i = 0; i + 1 < tok.size(); i++) c.push_back(std::stoi(tok[i]));
    if (dims == 0) dims = int(c.size());
    if (int(c.size()) != dims) throw fcc::Error(FCC_ERR_ARG, "ragged line in " + fname);
    nonzeros.emplace_back(DT(std::stod(tok.back())), CoOrdinate(c));
  }
  dimensionality = dims;
  shape_store.assign(size_t(dims), 0);
  for (auto &z : nonzeros)
    for (int i = 0; i < dims; i++)
      if (z.get_coords().get_index(i) > shape_store[i]) shape_store[i] = z.get_coords().get_index(i);
  shape = shape_store.data();
}

// Appends "shape line" then one "coords value" line per nonzero
// (read.hpp:108-142).
template <class DT> void Tensor<DT>::write(std::string fname) {
  std::ofstream file(fname, std::ios_base::app);
  for (int i = 0; i < dimensionality; i++) file << (shape ? shape[i] : 0) << " ";
  file << "\n";
  file.precision(17);
  for (auto &z : nonzeros) file << z.get_coords().to_string() << z.get_data() << "\n";
}

#endif
