// Host-side helpers shared by the library: thread-local error text and the raw
// binary array format of the reference (core/io.hpp:25-40: little-endian 4-byte
// elements, no header, element count = file bytes / 4).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace c2g {

// Record an error message for c2g_last_error() and return `code`.
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
const char* last_error();
void clear_error();

bool file_exists(const std::string& path);

// Read a whole file of 4-byte elements.  Returns C2G_OK, C2G_ERR_IO (missing or
// unreadable) or C2G_ERR_FORMAT (size not a multiple of 4).
int read_array4(const std::string& path, std::vector<int32_t>& out);
int read_array4(const std::string& path, std::vector<float>& out);

// Write `n` 4-byte elements (truncating the file).
int write_array4(const std::string& path, const void* data, size_t n);
int make_dir(const std::string& path);

// Check that vlist[V+1] is a row pointer: starts at 0, never decreases.
int check_rows(const std::vector<int32_t>& vlist);
// Check that vlist[V+1] is a CSR row pointer over E edges and elist ids are < V.
int check_csr(const std::vector<int32_t>& vlist, const std::vector<int32_t>& elist);

}  // namespace c2g
