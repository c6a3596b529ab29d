// tsg_mtx.h -- the Matrix Market reader's pieces shared by the host loader
// (tsg_mtx.cpp) and the device loader (tsg_load_mtx_device, tsg_api.cu).
#pragma once
#include <string>

#include "tilespgemm.h"

namespace tsg {

// value kinds of a coordinate file
enum MtxKind { MTX_REAL = 0, MTX_COMPLEX = 1, MTX_INTEGER = 2, MTX_PATTERN = 3 };

struct MtxHeader {
    long long M = 0, N = 0, NZ = 0;
    int kind = MTX_REAL;
    bool symm = false;        // symmetric or hermitian: mirrored
    size_t cursor = 0;        // just past the size line's NZ
    bool lines = false;       // the rest of the size line is blank
    size_t data = 0;          // first data line (when `lines`)
};

// The file's bytes with a '\n' appended; false if it cannot be read.
bool mtx_read_file(const char *path, std::string &out);
// Banner, comments and size line (mmio.h:400-496, :561-590 semantics).
tsg_status mtx_header(const std::string &text, MtxHeader &h);
// One non-blank data line [p, e): exactly one entry, or false.
bool mtx_line(const char *p, const char *e, int kind, long long &i, long long &j, double &v);

}  // namespace tsg
