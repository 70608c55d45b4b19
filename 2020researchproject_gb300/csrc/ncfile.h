// Minimal writer and reader of netCDF classic files (the CDF-1 format, or
// CDF-2 when offsets pass 2 GiB), for the reference-compatible export
// (src/ibm3d_export.c:16-253 writes through the netCDF library) and
// restart (src/ibm3d_init.c:45-224).  Fixed-size dimensions only, the
// types the export uses (char attributes, int, float and double
// variables), big-endian as the format requires.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ibm {

enum { NCT_CHAR = 2, NCT_INT = 4, NCT_FLOAT = 5, NCT_DOUBLE = 6 };

struct NcVar {
    std::string name;
    int type;
    std::vector<int> dims;                                     // dimension ids
    std::vector<std::pair<std::string, std::string>> atts;     // text attributes
    const void *data = nullptr;                                // host values (writer)
    long long begin = 0;                                       // file offset (reader)
};

struct NcFile {
    std::vector<std::pair<std::string, long long>> dims;
    std::vector<NcVar> vars;
};

// Writes `f` (values from each var's data pointer).  Returns false on an I/O error.
bool nc_write(const std::string &path, const NcFile &f);

// Reads the header of a classic file into `f` (var begins set); false if
// the file is not one.
bool nc_read_header(const std::string &path, NcFile &f);

// Reads variable `name` converted to double (float, double or int
// variables).  Returns false if it is missing or the file is short.
bool nc_read_var(const std::string &path, const NcFile &f, const std::string &name, std::vector<double> &out);

}  // namespace ibm
