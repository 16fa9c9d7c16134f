// Restart-vector text I/O in the reference's wf_self_as_guess.out format.
//
// Writer: calExcitedEnergy (src/minres.cpp:59-70) writes the vector's length on
// one line, then one line per determinant: the key as an unsigned decimal, a
// space, and the amplitude with 12 significant digits (ostream default float
// format after std::setprecision(12)).  Reader: readPsi (src/main.cpp:288-307)
// reads the length with "%u" and then "%llu %lf" pairs.
//
// Keys wider than 64 bits (two words, up to 128 spin orbitals) are written as
// the decimal value of the whole 128-bit key, so files of 64-bit systems are
// byte-for-byte the reference's.  The host functions need no GPU; the vector
// functions download or upload through the context stream.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"

namespace sfci {

static std::string u128_decimal(u64 lo, u64 hi) {
  unsigned __int128 v = ((unsigned __int128)hi << 64) | lo;
  if (v == 0) return "0";
  char buf[48];
  int p = 47;
  buf[p] = 0;
  while (v) {
    buf[--p] = (char)('0' + (int)(v % 10));
    v /= 10;
  }
  return std::string(buf + p);
}

// decimal string -> 128-bit key; false on a non-digit or overflow
static bool parse_u128(const std::string& s, u64& lo, u64& hi) {
  if (s.empty()) return false;
  unsigned __int128 v = 0;
  const unsigned __int128 lim = ~(unsigned __int128)0 / 10;
  for (char ch : s) {
    if (ch < '0' || ch > '9') return false;
    if (v > lim) return false;
    v *= 10;
    const unsigned d = (unsigned)(ch - '0');
    if (v > ~(unsigned __int128)0 - d) return false;
    v += d;
  }
  lo = (u64)v;
  hi = (u64)(v >> 64);
  return true;
}

int psi_write(const u64* keys, const double* amps, u64 n, int words, const char* path) {
  if (!path || (n && (!keys || !amps)) || (words != 1 && words != 2))
    return set_error(SFCI_ERR_ARG, "psi write: bad argument");
  std::ofstream f(path, std::ios::trunc);
  if (!f) return set_error(SFCI_ERR_IO, std::string("cannot open ") + path + " for writing");
  f << n << '\n';
  f << std::setprecision(12);
  for (u64 i = 0; i < n; ++i) {
    if (words == 1) f << keys[i];
    else f << u128_decimal(keys[2 * i], keys[2 * i + 1]);
    f << ' ' << amps[i] << '\n';
  }
  f.flush();
  if (!f) return set_error(SFCI_ERR_IO, std::string("write to ") + path + " failed");
  return SFCI_OK;
}

// reads the length into *len; with keys == nullptr it stops there
int psi_read(const char* path, int words, int num_orb, u64* keys, double* amps, u64 cap, u64* len) {
  if (!path || !len || (words != 1 && words != 2) || num_orb < 1 || num_orb > 64 * words)
    return set_error(SFCI_ERR_ARG, "psi read: bad argument");
  std::ifstream f(path);
  if (!f) return set_error(SFCI_ERR_IO, std::string("cannot open ") + path);
  std::string tok;
  if (!(f >> tok)) return set_error(SFCI_ERR_IO, std::string(path) + ": missing length line");
  u64 nlo = 0, nhi = 0;
  if (!parse_u128(tok, nlo, nhi) || nhi || nlo > 0xffffffffull)
    return set_error(SFCI_ERR_IO, std::string(path) + ": bad length '" + tok + "'");
  const u64 n = nlo;
  *len = n;
  if (!keys && !amps && cap == 0) return SFCI_OK;
  if (n > cap) return set_error(SFCI_ERR_CAPACITY, std::string(path) + " holds more determinants than the capacity");
  if (n && (!keys || !amps)) return set_error(SFCI_ERR_ARG, "psi read: null buffers");
  for (u64 i = 0; i < n; ++i) {
    std::string ks, as;
    if (!(f >> ks >> as)) return set_error(SFCI_ERR_IO, std::string(path) + ": truncated at entry " + std::to_string(i));
    u64 lo = 0, hi = 0;
    if (!parse_u128(ks, lo, hi)) return set_error(SFCI_ERR_IO, std::string(path) + ": bad key '" + ks + "'");
    const bool fits = num_orb >= 128 ? true
                      : num_orb >= 64 ? (num_orb == 64 ? hi == 0 : (hi >> (num_orb - 64)) == 0)
                                      : (hi == 0 && (lo >> num_orb) == 0);
    if (!fits) return set_error(SFCI_ERR_ARG, std::string(path) + ": key '" + ks + "' has bits beyond num_orb");
    errno = 0;
    char* endp = nullptr;
    const double a = std::strtod(as.c_str(), &endp);
    if (endp == as.c_str() || *endp || errno == ERANGE)
      return set_error(SFCI_ERR_IO, std::string(path) + ": bad amplitude '" + as + "'");
    if (words == 1) {
      keys[i] = lo;
    } else {
      keys[2 * i] = lo;
      keys[2 * i + 1] = hi;
    }
    amps[i] = a;
  }
  return SFCI_OK;
}

}  // namespace sfci

using namespace sfci;

extern "C" int sfci_psi_write(const uint64_t* keys, const double* amps, uint64_t n, int key_words,
                              const char* path) {
  return psi_write((const u64*)keys, amps, n, key_words, path);
}

extern "C" int sfci_psi_read(const char* path, int key_words, int num_orb, uint64_t* keys, double* amps,
                             uint64_t cap, uint64_t* len) {
  return psi_read(path, key_words, num_orb, (u64*)keys, amps, cap, (u64*)len);
}

extern "C" int sfci_vec_save(const sfci_vec* v, const char* path) {
  if (!v || !v->v.ctx) return set_error(SFCI_ERR_ARG, "null vector");
  u64 len = v->v.len;
  const int words = v->v.ctx->W;
  int st;
  std::vector<uint64_t> k(len * (u64)words + 1);
  std::vector<double> a(len + 1);
  uint64_t got = 0;
  if ((st = sfci_vec_download(v, k.data(), a.data(), len, &got))) return st;
  return psi_write((const u64*)k.data(), a.data(), got, words, path);
}

extern "C" int sfci_vec_load(sfci_vec* v, const char* path) {
  if (!v || !v->v.ctx) return set_error(SFCI_ERR_ARG, "null vector");
  const u64 cap = v->v.cap;
  const int words = v->v.ctx->W, num_orb = v->v.ctx->N;
  u64 len = 0;
  // length first, so that the buffers are sized by the file, not the capacity
  int st = psi_read(path, words, num_orb, nullptr, nullptr, 0, &len);
  if (st) return st;
  if (len > cap) return set_error(SFCI_ERR_CAPACITY, std::string(path) + " holds more determinants than the capacity");
  std::vector<uint64_t> k(len * (u64)words + 1);
  std::vector<double> a(len + 1);
  if ((st = psi_read(path, words, num_orb, (u64*)k.data(), a.data(), len, &len))) return st;
  return sfci_vec_upload(v, k.data(), a.data(), len);
}
