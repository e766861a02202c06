// GFmatrix restart files: the layout that save_gfprime writes and
// read_gfprime reads (VCA_AUX_FUNX.f90:486-697).  Host code only.
//
// The file holds one GFmatrix per spin-diagonal element, in the order of the
// reference's loops: ilat, jlat, ispin, iorb, jorb from the outer to the
// inner loop (VCA_AUX_FUNX.f90:627-641).  One GFmatrix is
//   Nstates, then per state: Nchan, then per channel: Nexc, Nexc complex
//   poles, Nexc complex weights
// (write_formatted / write_unformatted, :486-566).  Two encodings:
// * unformatted: one sequential record per element -- a 4-byte
//   little-endian byte count before and after the payload, integers as
//   4-byte little-endian, complex numbers as two little-endian IEEE doubles
//   (the record layout of sequential unformatted files on little-endian
//   hosts; a user-defined derived-type write adds nothing between its
//   items);
// * formatted: list-directed text, one line per element (the child writes of
//   a derived-type write do not start new records), complex numbers as
//   (re,im) with 17 significant digits, which reads back bit-exact.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

struct GfmTable {
  // flattened in file order
  std::vector<int32_t> nstates;  // [nelem]
  std::vector<int32_t> nchan;    // [sum nstates]
  std::vector<int32_t> nexc;     // [sum nchan]
  std::vector<double> poles;     // [2 * sum nexc] (re, im)
  std::vector<double> weights;   // [2 * sum nexc]
};

// counts consistent with one another and with the data lengths
bool gfm_consistent(const GfmTable& t, std::string& err);
// 0 on success, -1 with a message in err
int gfm_write(const std::string& path, bool formatted, const GfmTable& t, std::string& err);
// reads nelem elements; data after them is ignored, as the reference's
// reader ignores it
int gfm_read(const std::string& path, bool formatted, int64_t nelem, GfmTable& t, std::string& err);
