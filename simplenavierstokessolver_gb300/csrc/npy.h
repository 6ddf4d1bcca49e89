// NPY files as the reference's save/restart path writes and reads them
// (src/fileio.c:81-345 over src/simple_npyio.c): format 1.0 (2.0 when the
// dictionary exceeds 65471 bytes), dictionary without spaces
// "{'descr':'float64','fortran_order':False,'shape':(jtot,itot+2,)}",
// space padding and a final newline to a multiple of 64 bytes, little-endian
// data in C order. Host code only.
#pragma once

#include <cstddef>
#include <string>

namespace sns {

// dtype is the reference's descriptor text: "'float64'" or "'int32'"
int npy_write(const char *path, const char *dtype, int ndim, const size_t *shape, const void *data, size_t nbytes,
              std::string *err);
// reads a C-order array whose shape must equal `shape` and whose descriptor
// must be the given one or its numpy spelling ('<f8', '<i4'); data gets nbytes
int npy_read(const char *path, const char *dtype, int ndim, const size_t *shape, void *data, size_t nbytes,
             std::string *err);
// mkdir -p
int make_dirs(const char *path, std::string *err);

}  // namespace sns
