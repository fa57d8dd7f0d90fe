// Field tables on the host: the reference's text files (Data/ic.txt,
// Data/moore_ic.txt, finalField.txt: one line per site in linear order,
// whitespace-separated columns) and a binary form of the same table.
//
// The reference reads them with `ic >> value` one token at a time
// (evolution.cpp:107-129), several seconds per million sites.  Here the whole
// file is read at once and parsed with std::from_chars on every host core, each
// thread taking a run of whole lines; values keep their exact doubles.
//
// Binary form ("AXIONSB1"): the 8-byte magic, int64 rows, int64 cols, then
// rows*cols little-endian doubles, row-major (the text's order).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace axh {

// Reads `rows` rows of `cols` values from a text or binary table (chosen by the
// file's first bytes) into dst[c * rows + r] (column-major, the lattice
// layout).  Throws std::runtime_error naming the file and line on a short file,
// a wrong column count, an unparsable or non-finite value, or trailing data.
void read_table(const std::string& path, int cols, int64_t rows, std::vector<double>& dst);

// Writes the column-major table src[c * rows + r] as text, one line per row,
// values separated by one space and printed as `ostream << double` prints them
// at `digits` significant digits (%g), in parallel.
void write_table_text(const std::string& path, int cols, int64_t rows, const double* src, int digits);

// Writes the column-major table as the binary form.
void write_table_bin(const std::string& path, int cols, int64_t rows, const double* src);

// True when the file starts with the binary magic.
bool is_binary_table(const std::string& path);

}  // namespace axh
