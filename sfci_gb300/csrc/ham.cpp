// _IN integral file -> dense spin-blocked integral tables.
//
// The reference reader (ReadElements, src/functions.cpp:297-395) reads seven
// count-prefixed groups of "coeff m n p q" lines, shifts every index by -2 and
// routes each entry: the all-zero entry is the core energy (:322-325); p = q = 0
// entries are one-body, diagonal (:326-334) or not (:336-344); two-body entries
// with (m==n && p==q) or (m==q && n==p) are diagonal (:354-359), all others go
// to per-occupied-pair lists (:360-378).  It stops after the first group whose
// count is 1 (:392).
//
// This loader keeps the same grouping, index shift and early stop, but stores
// values in dense tables addressed by spin orbitals instead of lists, so that
// the device excitation generator can look any matrix element up directly.
// The tables assume what convert_fcidump.py guarantees: (mn|pq) = (nm|pq) =
// (mn|qp) within a spin block, every entry once.  An entry that contradicts
// an earlier one, a repeated entry, or a spin-mixing (m,n) pair is rejected
// rather than silently reinterpreted.
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "internal.h"

namespace sfci {

static inline int spair(int i, int j) { return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

int load_in_file(const char* path, int N, HamHost& H, std::string& err) {
  FILE* fp = fopen(path, "rb");
  if (!fp) {
    err = std::string("cannot open integral file: ") + path;
    return SFCI_ERR_IO;
  }
  std::string buf;
  {
    fseek(fp, 0, SEEK_END);
    long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    if (sz > 0 && fread(&buf[0], 1, (size_t)sz, fp) != (size_t)sz) {
      fclose(fp);
      err = "short read on integral file";
      return SFCI_ERR_IO;
    }
    fclose(fp);
  }
  const int M = N / 2;
  const int P = M * (M + 1) / 2;
  H.M = M;
  H.N = N;
  H.P = P;
  H.ecore = 0.0;
  H.h1.assign((size_t)2 * M * M, 0.0);
  H.V.assign((size_t)4 * P * P, 0.0);
  std::vector<uint8_t> vset((size_t)4 * P * P, 0), hset((size_t)2 * M * M, 0);
  std::vector<uint64_t> seen2(((size_t)N * N * N * N + 63) / 64, 0);
  std::vector<uint64_t> seen1(((size_t)N * N + 63) / 64, 0);

  const char* s = buf.c_str();
  char* e = nullptr;
  H.n_two = H.n_one = 0;
  for (int g = 0; g < 7; ++g) {
    long cnt = strtol(s, &e, 10);
    if (e == s) {
      if (g == 0) {
        err = "integral file has no group count";
        return SFCI_ERR_IO;
      }
      break;  // the reference's fscanf leaves missing trailing groups empty
    }
    s = e;
    for (long i = 0; i < cnt; ++i) {
      double coeff = strtod(s, &e);
      if (e == s) { err = "malformed coefficient in integral file"; return SFCI_ERR_IO; }
      s = e;
      long idx[4];
      for (int t = 0; t < 4; ++t) {
        idx[t] = strtol(s, &e, 10);
        if (e == s) { err = "malformed index in integral file"; return SFCI_ERR_IO; }
        s = e;
      }
      long m = idx[0], n = idx[1], p = idx[2], q = idx[3];
      if (p == 0 && q == 0) {
        if (m == n && m == 0) {
          H.ecore = coeff;
          continue;
        }
        long a = m - 2, b = n - 2;
        if (a < 0 || b < 0 || a >= N || b >= N) {
          err = "one-body index out of range for num_orb";
          return SFCI_ERR_ARG;
        }
        if ((a & 1) != (b & 1)) { err = "spin-mixing one-body entry"; return SFCI_ERR_UNSUPPORTED; }
        size_t bit = (size_t)a * N + b;
        if (seen1[bit >> 6] >> (bit & 63) & 1) { err = "repeated one-body entry"; return SFCI_ERR_UNSUPPORTED; }
        seen1[bit >> 6] |= 1ull << (bit & 63);
        size_t slot = ((size_t)(a & 1) * M + (a >> 1)) * M + (b >> 1);
        H.h1[slot] = coeff;
        hset[slot] = 1;
        H.n_one++;
      } else {
        long a = m - 2, b = n - 2, c = p - 2, d = q - 2;
        if (a < 0 || b < 0 || c < 0 || d < 0 || a >= N || b >= N || c >= N || d >= N) {
          err = "two-body index out of range for num_orb";
          return SFCI_ERR_ARG;
        }
        if ((a & 1) != (b & 1) || (c & 1) != (d & 1)) {
          err = "spin-mixing two-body entry";
          return SFCI_ERR_UNSUPPORTED;
        }
        size_t bit = (((size_t)a * N + b) * N + c) * N + d;
        if (seen2[bit >> 6] >> (bit & 63) & 1) { err = "repeated two-body entry"; return SFCI_ERR_UNSUPPORTED; }
        seen2[bit >> 6] |= 1ull << (bit & 63);
        int blk = (int)((a & 1) * 2 + (c & 1));
        size_t slot = ((size_t)blk * P + spair((int)(a >> 1), (int)(b >> 1))) * P +
                      spair((int)(c >> 1), (int)(d >> 1));
        if (vset[slot] && H.V[slot] != coeff) {
          char msg[160];
          snprintf(msg, sizeof msg, "two-body entry (%ld %ld %ld %ld) contradicts a symmetric partner",
                   m, n, p, q);
          err = msg;
          return SFCI_ERR_UNSUPPORTED;
        }
        H.V[slot] = coeff;
        vset[slot] = 1;
        H.n_two++;
      }
    }
    if (cnt == 1) break;  // src/functions.cpp:392
  }
  return SFCI_OK;
}

}  // namespace sfci
