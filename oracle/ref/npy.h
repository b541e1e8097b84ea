// Minimal .npy reader/writer (little-endian, C order, '<f8' and '<i4' only).
// Test infrastructure for the oracle tools; not part of the product library.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace npy {

struct Array {
  std::string dtype;             // "<f8" or "<i4"
  std::vector<long> shape;
  std::vector<unsigned char> bytes;
  long size() const { long n = 1; for (long s : shape) n *= s; return n; }
  const double* f8() const { return reinterpret_cast<const double*>(bytes.data()); }
  const int32_t* i4() const { return reinterpret_cast<const int32_t*>(bytes.data()); }
};

inline Array load(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + path);
  char magic[8];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "\x93NUMPY", 6) != 0)
    throw std::runtime_error("not an npy file: " + path);
  uint32_t hlen = 0;
  if (magic[6] == 1) { uint16_t h16; if (std::fread(&h16, 2, 1, f) != 1) throw std::runtime_error("short"); hlen = h16; }
  else { if (std::fread(&hlen, 4, 1, f) != 1) throw std::runtime_error("short"); }
  std::string header(hlen, ' ');
  if (std::fread(&header[0], 1, hlen, f) != hlen) throw std::runtime_error("short header");
  Array a;
  size_t d = header.find("'descr':");
  size_t q1 = header.find('\'', d + 8), q2 = header.find('\'', q1 + 1);
  a.dtype = header.substr(q1 + 1, q2 - q1 - 1);
  if (header.find("'fortran_order': True") != std::string::npos)
    throw std::runtime_error("fortran order unsupported: " + path);
  size_t p1 = header.find('(', header.find("'shape':")), p2 = header.find(')', p1);
  std::string sh = header.substr(p1 + 1, p2 - p1 - 1);
  size_t pos = 0;
  while (pos < sh.size()) {
    size_t c = sh.find(',', pos);
    std::string tok = sh.substr(pos, c == std::string::npos ? std::string::npos : c - pos);
    if (tok.find_first_of("0123456789") != std::string::npos) a.shape.push_back(std::stol(tok));
    if (c == std::string::npos) break;
    pos = c + 1;
  }
  size_t esize = (a.dtype == "<f8") ? 8 : (a.dtype == "<i4") ? 4 : 0;
  if (!esize) throw std::runtime_error("unsupported dtype " + a.dtype + " in " + path);
  a.bytes.resize(a.size() * esize);
  if (std::fread(a.bytes.data(), 1, a.bytes.size(), f) != a.bytes.size())
    throw std::runtime_error("short data in " + path);
  std::fclose(f);
  return a;
}

inline void save(const std::string& path, const void* data, const std::string& dtype,
                 const std::vector<long>& shape) {
  std::string sh = "(";
  for (size_t i = 0; i < shape.size(); i++) sh += std::to_string(shape[i]) + ",";
  if (shape.size() > 1) sh.pop_back();
  sh += ")";
  std::string header = "{'descr': '" + dtype + "', 'fortran_order': False, 'shape': " + sh + ", }";
  size_t total = 10 + header.size() + 1;
  header += std::string((64 - total % 64) % 64, ' ') + "\n";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fwrite("\x93NUMPY\x01\x00", 1, 8, f);
  uint16_t hl = (uint16_t)header.size();
  std::fwrite(&hl, 2, 1, f);
  std::fwrite(header.data(), 1, header.size(), f);
  long n = 1;
  for (long s : shape) n *= s;
  std::fwrite(data, dtype == "<f8" ? 8 : 4, n, f);
  std::fclose(f);
}

}  // namespace npy
