// `sfci` — process-level drop-in for the reference binary (src/main.cpp:154-280):
// reads `sfci.input` from the working directory (key=value lines, keys of
// src/main.cpp:58-124), loads the _IN integrals, prints the parameter summary
// and E_hf, runs the truncated Lanczos ground-state solve on the GPU and prints
// the reference's key lines (gsaes energy, final e, SFCI time).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/sfci_gb300.h"

struct Params {
  unsigned long long Nd = 200000, init_hf_lo = 0, init_hf_hi = 0;
  int Nl = 0, num_restart = 0, num_orb = 0, num_e = 0, num_thread = 0;
  unsigned long long bucket_unit = 60000;
  std::string filename, task, init_hf_text;
  bool init_hf_ok = false;
  double coeff_cut = 1e-5, target_E = 0.0;
};

// decimal string -> 128-bit value; false for other characters, no digits or
// a value beyond 128 bits
static bool parse_u128(const std::string& s, unsigned long long& lo, unsigned long long& hi) {
  const unsigned __int128 top = ~(unsigned __int128)0;
  unsigned __int128 v = 0;
  bool any = false;
  for (char ch : s) {
    if (ch < '0' || ch > '9') {
      if (ch == ' ' || ch == '\r' || ch == '\t') continue;
      return false;
    }
    const unsigned d = (unsigned)(ch - '0');
    if (v > (top - d) / 10) return false;
    v = v * 10 + d;
    any = true;
  }
  lo = (unsigned long long)v;
  hi = (unsigned long long)(v >> 64);
  return any;
}

// the determinant has no bit at or above num_orb
static bool fits_orbitals(unsigned long long lo, unsigned long long hi, int num_orb) {
  if (num_orb >= 128) return true;
  if (num_orb >= 64) return (hi >> (num_orb - 64)) == 0;
  return hi == 0 && (lo >> num_orb) == 0;
}

static void parse(Params& p, const std::string& key, const std::string& val) {
  // like the reference: no trimming, unknown keys ignored (src/main.cpp:58-124)
  auto echo = [&](const std::string& v) { printf("using input %s=%s\n", key.c_str(), v.c_str()); };
  if (key == "num_thread") { p.num_thread = std::stoi(val); echo(val); }
  else if (key == "Nd") { p.Nd = std::stoull(val); echo(val); }
  else if (key == "Nl") { p.Nl = std::stoi(val); echo(val); }
  else if (key == "num_restart") { p.num_restart = std::stoi(val); echo(val); }
  else if (key == "num_orb") { p.num_orb = std::stoi(val); echo(val); }
  else if (key == "num_e") { p.num_e = std::stoi(val); echo(val); }
  else if (key == "filename") { p.filename = val; echo(val); }
  else if (key == "coeff_cut") { p.coeff_cut = std::stod(val); echo(val); }
  else if (key == "bucket_unit") { p.bucket_unit = std::stoull(val); echo(val); }
  else if (key == "init_hf") { p.init_hf_text = val; p.init_hf_ok = parse_u128(val, p.init_hf_lo, p.init_hf_hi); echo(val); }
  else if (key == "task") { p.task = val; echo(val); }
  else if (key == "target_E") { p.target_E = std::stod(val); echo(val); }
}

int main(int argc, char** argv) {
  const char* input = argc > 1 ? argv[1] : "sfci.input";
  Params p;
  std::ifstream f(input);
  if (f.is_open()) {
    std::string raw;
    while (std::getline(f, raw)) {
      auto pos = raw.find('=');
      if (pos == std::string::npos) continue;  // the reference would misparse; skip instead
      const std::string key = raw.substr(0, pos), val = raw.substr(pos + 1);
      try {
        parse(p, key, val);
      } catch (const std::exception&) {  // std::stoi and friends: not a number, or out of range
        fprintf(stderr, "sfci: bad value for %s: %s\n", key.c_str(), val.c_str());
        return 1;
      }
    }
  }
  if (p.task == "ground") {
    if (!p.init_hf_ok) {
      fprintf(stderr, "sfci: init_hf must be a decimal integer below 2^128: %s\n", p.init_hf_text.c_str());
      return 1;
    }
    // (a num_orb outside [1, 128] is reported by the context set-up)
    if (p.num_orb > 0 && p.num_orb <= 128 && !fits_orbitals(p.init_hf_lo, p.init_hf_hi, p.num_orb)) {
      fprintf(stderr, "sfci: init_hf %s sets a spin orbital at or above num_orb=%d\n", p.init_hf_text.c_str(),
              p.num_orb);
      return 1;
    }
  }
  sfci_opts o{};
  o.Nd = p.Nd;
  o.hpsi_cap = 60000000;
  o.coeff_cut = 1e-5;  // src/main.cpp:196 overrides coeff_cut
  o.verbose = 1;
  sfci_ctx* ctx = nullptr;
  int st = sfci_ctx_create(p.filename.c_str(), p.num_orb, p.num_e, &o, &ctx);
  if (st) {
    fprintf(stderr, "sfci: %s: %s\n", sfci_status_name(st), sfci_last_error());
    return 1;
  }
  printf("integrals loaded\n");
  int W = sfci_key_words(ctx);
  printf("\n*****************parameters summary*****************\n");
  printf("input file:%s\norbital num:%d\nelectron num:%d\nNd:%llu\n", p.filename.c_str(), p.num_orb, p.num_e,
         (unsigned long long)p.Nd);
  printf("SpMSpV final result cut:%g\n", 1e-5);
  printf("\n****************************************************\n");
  int rc = 0;
  if (p.task == "ground") {
    uint64_t key[2] = {(uint64_t)p.init_hf_lo, (uint64_t)p.init_hf_hi};
    double ehf = 0.0;
    st = sfci_diag_elements(ctx, key, 1, &ehf);
    if (!st) printf("E_hf:%.12f\n", ehf);
    sfci_vec* v = nullptr;
    if (!st) st = sfci_vec_create(ctx, p.Nd, &v);
    double one = 1.0;
    if (!st) st = sfci_vec_upload(v, key, &one, 1);
    (void)W;
    auto t1 = std::chrono::system_clock::now();
    std::vector<double> en(p.num_restart > 0 ? p.num_restart : 1);
    double fe = 0.0;
    if (!st) st = sfci_lanczos_ground(ctx, v, p.Nl, p.num_restart, en.data(), &fe);
    auto t2 = std::chrono::system_clock::now();
    if (st) {
      fprintf(stderr, "sfci: %s: %s\n", sfci_status_name(st), sfci_last_error());
      rc = 1;
    } else {
      printf("SFCI time: %.6f\n", std::chrono::duration<double>(t2 - t1).count());
    }
    sfci_vec_destroy(v);
  } else if (p.task == "excited") {
    // src/main.cpp:235-242: an empty stub in the reference
  }
  sfci_ctx_destroy(ctx);
  return rc;
}
