// Oracle restatement of the SFCI hot path — TEST INFRASTRUCTURE ONLY.
//
// A C++/OpenMP restatement of the reference algorithm, used by the tests as the
// oracle and by bench.py as the timed CPU baseline ("port").  Nothing in the
// product links it.  It follows the reference function by function, with each
// step citing the reference line it restates, and generalises the determinant
// type to 128 bits so that it also covers systems beyond 64 spin orbitals
// (the reference stops at 64, src/main.cpp:84-85).  Differences that do not
// change results: buffers grow instead of having fixed capacities (the
// reference overflows them, src/functions.cpp:566,616 and src/bitstr.cpp:311),
// buckets use a hash of the whole determinant instead of the alpha-string rank
// (src/bitstr.cpp:74-131, whose nck table overflows past 64 spin orbitals), and
// the sorts are std::sort/std::stable_sort instead of the hand-written introsort
// (src/introsort.cpp).  Pinned against the compiled reference through the
// golden fixtures of tests/golden.
#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

typedef unsigned long long u64;
typedef unsigned __int128 u128;

namespace {

struct Ham {
  int N = 0, ne = 0;
  double constant = 0.0;
  // src/all.h:105-125: OO lists per occupied pair index n + N*q, O lists per n
  std::vector<std::vector<std::array<unsigned char, 4>>> OO;
  std::vector<std::vector<double>> OO_c;
  std::vector<std::vector<std::array<unsigned char, 2>>> O;
  std::vector<std::vector<double>> O_c;
  std::vector<std::array<unsigned char, 4>> OO_diag;
  std::vector<double> OO_diag_c;
  std::vector<std::array<unsigned char, 2>> O_diag;
  std::vector<double> O_diag_c;
};

Ham H;
unsigned g_Nd = 200000;
int g_threads = 1;
double kCut = 1e-5;  // SpMSpVFinalResCut, src/main.cpp:196 (settable: a negative cut keeps every merged term)

// ReadElements, src/functions.cpp:297-395
bool read_elements(const char* path) {
  FILE* fp = fopen(path, "r");
  if (!fp) return false;
  H.constant = 0.0;
  for (int g = 0; g < 7; ++g) {
    int num = 0;
    if (fscanf(fp, "%d", &num) != 1) break;
    for (int i = 0; i < num; ++i) {
      double c;
      int m, n, p, q;
      if (fscanf(fp, "%lf %d %d %d %d", &c, &m, &n, &p, &q) != 5) {
        fclose(fp);
        return false;
      }
      if (p == 0 && q == 0) {
        if (m == n) {
          if (m == 0) H.constant = c;                       // :322-325
          else { H.O_diag.push_back({(unsigned char)(m - 2), (unsigned char)(n - 2)}); H.O_diag_c.push_back(c); }
        } else {                                             // :336-344, indexed by the annihilated orbital
          H.O[n - 2].push_back({(unsigned char)(m - 2), (unsigned char)(n - 2)});
          H.O_c[n - 2].push_back(c);
        }
      } else {
        std::array<unsigned char, 4> t = {(unsigned char)(m - 2), (unsigned char)(n - 2), (unsigned char)(p - 2),
                                          (unsigned char)(q - 2)};
        if ((t[0] == t[1] && t[2] == t[3]) || (t[0] == t[3] && t[2] == t[1])) {  // :354-359
          H.OO_diag.push_back(t);
          H.OO_diag_c.push_back(c);
        } else if (!(m == n || n == p || p == q || m == q)) {                    // :362-369
          if (t[1] < t[3]) {
            H.OO[t[1] + H.N * t[3]].push_back(t);
            H.OO_c[t[1] + H.N * t[3]].push_back(c);
          }
        } else {                                                                 // :371-378
          int idx = t[1] < t[3] ? t[1] + H.N * t[3] : t[3] + H.N * t[1];
          H.OO[idx].push_back(t);
          H.OO_c[idx].push_back(c);
        }
      }
    }
    if (num == 1) break;  // :392
  }
  fclose(fp);
  return true;
}

// ---- determinant helpers, generic over the key type ---------------------------

template <class D> inline D bit(int b) { return (D)1 << b; }
inline int popc(u64 x) { return __builtin_popcountll(x); }
inline int popc(u128 x) { return __builtin_popcountll((u64)x) + __builtin_popcountll((u64)(x >> 64)); }

// signCal_bit, src/bitstr.cpp:133-160: parity of occupied orbitals strictly between p < q
template <class D> inline double sign_between(D ref, int p, int q) {
  const int nb = (int)sizeof(D) * 8;
  D t = ref;
  t >>= (p + 1);
  t <<= (p + 1);
  if (nb - q >= nb) t = 0; else t <<= (nb - q);
  return (popc(t) & 1) ? -1.0 : 1.0;
}
template <class D> inline double sgn(D ref, int a, int b) { return a < b ? sign_between(ref, a, b) : sign_between(ref, b, a); }

inline u64 mix64(u64 z) {
  z ^= z >> 30; z *= 0xbf58476d1ce4e5b9ull;
  z ^= z >> 27; z *= 0x94d049bb133111ebull;
  z ^= z >> 31;
  return z;
}
inline u64 hash_det(u64 d) { return mix64(d); }
inline u64 hash_det(u128 d) { return mix64((u64)d) ^ mix64((u64)(d >> 64) + 0x9e3779b97f4a7c15ull); }

// OffDiagGen_bit / OffDiagGen_bit_e (src/bitstr.cpp:162-302, :304-431): every
// emitted term of one determinant, in the reference's order, into `emit`.
template <class D, class F> void off_diag_gen(D reff, double coeff, F&& emit) {
  const D one = 1;
  int occ[128];
  int pos = 0;
  for (int i = 0; i < H.N; ++i)
    if (reff & (one << i)) occ[pos++] = i;                                      // :175-182
  const int ne = pos;
  for (int i = 0; i < ne; i++)
    for (int j = i + 1; j < ne; j++) {                                          // :185-190
      unsigned idx = occ[i] + occ[j] * H.N;
      const auto& L = H.OO[idx];
      const auto& Lc = H.OO_c[idx];
      for (size_t k = 0; k < L.size(); k++) {
        D start = reff;
        int m = L[k][0], n = L[k][1], p = L[k][2], q = L[k][3];
        bool m_free = !(reff & (one << m)), p_free = !(reff & (one << p));
        if (m != n && n != p && p != q && m != q && m_free && p_free) {         // :207-227
          double s = sgn(start, p, q);
          start = start - (one << q) + (one << p);
          s *= sgn(start, m, n);
          start = start - (one << n) + (one << m);
          emit(start, coeff * s * Lc[k]);
        } else if (m != n && n != p && p == q && q != m && m_free) {           // :230-246
          double s = sgn(start, m, n);
          start = start - (one << n) + (one << m);
          emit(start, coeff * s * Lc[k]);
        } else if (m != n && n == p && p != q && q != m && m_free) {           // :248-262
          double s = sgn(start, q, m);
          start = start - (one << q) + (one << m);
          emit(start, -coeff * s * Lc[k]);
        }
      }
    }
  for (int i = 0; i < ne; i++) {                                                // :269-300
    const auto& L = H.O[occ[i]];
    const auto& Lc = H.O_c[occ[i]];
    for (size_t j = 0; j < L.size(); j++) {
      D start = reff;
      int m = L[j][0], n = L[j][1];
      if (!(reff & (one << m))) {
        double s = sgn(start, m, n);
        start = start - (one << n) + (one << m);
        emit(start, coeff * s * Lc[j]);
      }
    }
  }
}

// DiagCal_bit, src/bitstr.cpp:433-476
template <class D> double diag_cal(D reff) {
  const D one = 1;
  double sum = H.constant;
  for (size_t i = 0; i < H.O_diag.size(); i++)
    if (reff & (one << H.O_diag[i][1])) sum += H.O_diag_c[i];
  for (size_t i = 0; i < H.OO_diag.size(); i++) {
    int m = H.OO_diag[i][0], n = H.OO_diag[i][1], p = H.OO_diag[i][2], q = H.OO_diag[i][3];
    if ((reff & (one << n)) && (reff & (one << q))) {
      if (m == n && p == q) sum += 0.5 * H.OO_diag_c[i];
      else if (m == q && n == p) sum -= 0.5 * H.OO_diag_c[i];
    }
  }
  return sum;
}

template <class D> struct Term {
  D k;
  double a;
};
template <class D> inline bool by_key(const Term<D>& x, const Term<D>& y) { return x.k < y.k; }
template <class D> inline bool by_abs(const Term<D>& x, const Term<D>& y) { return std::fabs(x.a) < std::fabs(y.a); }

// merge_bucket, src/functions.cpp:429-464 (key-sorted input, in place)
template <class D> size_t merge_runs(std::vector<Term<D>>& b, size_t n) {
  if (n <= 1) return n;
  size_t m = 0;
  D pk = b[0].k;
  double pa = b[0].a;
  for (size_t i = 1; i < n; ++i) {
    if (pk != b[i].k) {
      b[m++] = {pk, pa};
      pk = b[i].k;
      pa = b[i].a;
    } else {
      pa += b[i].a;
    }
  }
  b[m++] = {pk, pa};
  return m;
}

// dynVec::dot, src/all.h:317-351
template <class D> double dot_sorted(const Term<D>* x, size_t nx, const Term<D>* y, size_t ny) {
  size_t i = 0, j = 0;
  double s = 0.0;
  while (i < nx && j < ny) {
    if (x[i].k < y[j].k) ++i;
    else if (x[i].k > y[j].k) ++j;
    else s += x[i++].a * y[j++].a;
  }
  return s;
}

// SpMVMtply_bucket, src/functions.cpp:511-804
template <class D>
void spmspv(const std::vector<Term<D>>& in_o, size_t out_cap, double lambda, double coeff, std::vector<Term<D>>& out,
            double* diag) {
  out.clear();
  if (in_o.empty()) return;                                                       // :529-533
  std::vector<Term<D>> in = in_o;
  std::stable_sort(in.begin(), in.end(), by_abs<D>);                                // :535-538
  size_t st = in.size() < g_Nd ? 0 : in.size() - g_Nd;                              // :549
  const int T = g_threads;
  const size_t nb = (size_t)T * 64;
  auto bucket_of = [nb](D k) { return (size_t)(hash_det(k) % nb); };
  // bucketed, key-sorted copy of the truncated input (for the exact <v|H|v>, :577-605)
  std::vector<std::vector<Term<D>>> in_b(nb);
  for (size_t i = st; i < in.size(); ++i) in_b[bucket_of(in[i].k)].push_back(in[i]);
  for (auto& b : in_b) std::sort(b.begin(), b.end(), by_key<D>);
  // OMP region 1: generation into per-(thread, bucket) buffers (:623-639)
  std::vector<std::vector<Term<D>>> res((size_t)T * nb);
#pragma omp parallel num_threads(T)
  {
    const int tid = omp_get_thread_num();
#pragma omp for schedule(static, 25)
    for (long long i = (long long)st; i < (long long)in.size(); ++i) {
      const D bi = in[i].k;
      const double t = coeff * in[i].a;
      off_diag_gen<D>(bi, t, [&](D k, double a) { res[tid + (size_t)T * bucket_of(k)].push_back({k, a}); });
      res[tid + (size_t)T * bucket_of(bi)].push_back({bi, (diag_cal<D>(bi) - lambda) * t});
    }
  }
  // OMP region 2: per bucket concat + sort + merge + partial dot (:646-731)
  std::vector<std::vector<Term<D>>> local(nb);
  double alpha = 0.0;
#pragma omp parallel for schedule(dynamic) num_threads(T) reduction(+ : alpha)
  for (long long b = 0; b < (long long)nb; ++b) {
    auto& L = local[b];
    size_t tot = 0;
    for (int j = 0; j < T; ++j) tot += res[j + (size_t)T * b].size();
    L.reserve(tot);
    for (int j = 0; j < T; ++j) {
      auto& r = res[j + (size_t)T * b];
      L.insert(L.end(), r.begin(), r.end());
      std::vector<Term<D>>().swap(r);
    }
    std::sort(L.begin(), L.end(), by_key<D>);
    L.resize(merge_runs(L, L.size()));
    alpha += dot_sorted(L.data(), L.size(), in_b[b].data(), in_b[b].size());
  }
  *diag = alpha;                                                                  // :739
  // serial cut + top-cap + key sort (:741-793)
  std::vector<Term<D>> fin;
  for (auto& L : local)
    for (auto& t : L)
      if (std::fabs(t.a) > kCut) fin.push_back(t);
  std::stable_sort(fin.begin(), fin.end(), by_abs<D>);
  size_t s0 = fin.size() < out_cap ? 0 : fin.size() - out_cap;
  out.assign(fin.begin() + s0, fin.end());
  std::sort(out.begin(), out.end(), by_key<D>);
}

// calc_energy, src/functions.cpp:1272-1313
template <class D> double energy(const std::vector<Term<D>>& psi) {
  std::unordered_map<u64, std::vector<std::pair<D, double>>> pos;
  pos.reserve(psi.size());
  for (auto& t : psi) pos[hash_det(t.k)].push_back({t.k, t.a});
  double e = 0.0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : e) schedule(dynamic, 16)
  for (long long i = 0; i < (long long)psi.size(); ++i) {
    const D d = psi[i].k;
    double ei = psi[i].a * diag_cal<D>(d);
    off_diag_gen<D>(d, 1.0, [&](D k, double a) {
      auto it = pos.find(hash_det(k));
      if (it == pos.end()) return;
      for (auto& kv : it->second)
        if (kv.first == k) ei += a * kv.second;
    });
    e += psi[i].a * ei;
  }
  return e;
}

// addTwo, src/all.h:407-480
template <class D> void add_two(std::vector<Term<D>>& v, size_t cap, const std::vector<Term<D>>& w, double a) {
  std::vector<Term<D>> t;
  t.reserve(v.size() + w.size());
  size_t i = 0, j = 0;
  while (i < v.size() && j < w.size()) {
    if (v[i].k < w[j].k) t.push_back(v[i++]);
    else { t.push_back({w[j].k, a * w[j].a}); ++j; }
  }
  while (i < v.size()) t.push_back(v[i++]);
  while (j < w.size()) { t.push_back({w[j].k, a * w[j].a}); ++j; }
  size_t m = merge_runs(t, t.size());
  t.resize(m);
  std::stable_sort(t.begin(), t.end(), by_abs<D>);
  size_t st = m < cap ? 0 : m - cap;
  v.assign(t.begin() + st, t.end());
  std::sort(v.begin(), v.end(), by_key<D>);
}

// addThree, src/all.h:482-608 (cap = global Nd, |a| > 1e-14)
template <class D>
void add_three(std::vector<Term<D>>& v, const std::vector<Term<D>>& x, const std::vector<Term<D>>& y,
               const std::vector<Term<D>>& z, double a, double b, double c) {
  std::vector<Term<D>> t;
  t.reserve(x.size() + y.size() + z.size());
  size_t ix = 0, iy = 0, iz = 0;
  while (ix < x.size() && iy < y.size() && iz < z.size()) {
    D m = std::min(x[ix].k, std::min(y[iy].k, z[iz].k));
    if (m == x[ix].k) { t.push_back({x[ix].k, a * x[ix].a}); ++ix; }
    else if (m == y[iy].k) { t.push_back({y[iy].k, b * y[iy].a}); ++iy; }
    else { t.push_back({z[iz].k, c * z[iz].a}); ++iz; }
  }
  while (ix < x.size() && iy < y.size()) {
    if (x[ix].k < y[iy].k) { t.push_back({x[ix].k, a * x[ix].a}); ++ix; }
    else { t.push_back({y[iy].k, b * y[iy].a}); ++iy; }
  }
  while (ix < x.size() && iz < z.size()) {
    if (x[ix].k < z[iz].k) { t.push_back({x[ix].k, a * x[ix].a}); ++ix; }
    else { t.push_back({z[iz].k, c * z[iz].a}); ++iz; }
  }
  while (iz < z.size() && iy < y.size()) {
    if (y[iy].k < z[iz].k) { t.push_back({y[iy].k, b * y[iy].a}); ++iy; }
    else { t.push_back({z[iz].k, c * z[iz].a}); ++iz; }
  }
  while (ix < x.size()) { t.push_back({x[ix].k, a * x[ix].a}); ++ix; }
  while (iy < y.size()) { t.push_back({y[iy].k, b * y[iy].a}); ++iy; }
  while (iz < z.size()) { t.push_back({z[iz].k, c * z[iz].a}); ++iz; }
  size_t m = merge_runs(t, t.size());
  t.resize(m);
  std::stable_sort(t.begin(), t.end(), by_abs<D>);
  size_t st = m < g_Nd ? 0 : m - g_Nd;
  v.clear();
  for (size_t i = st; i < m; ++i)
    if (std::fabs(t[i].a) > 1e-14) v.push_back(t[i]);
  std::sort(v.begin(), v.end(), by_key<D>);
}

// shrinkFrom, src/all.h:281-299
template <class D> void shrink_from(std::vector<Term<D>>& dst, size_t cap, std::vector<Term<D>> src) {
  std::stable_sort(src.begin(), src.end(), by_abs<D>);
  size_t st = src.size() < cap ? 0 : src.size() - cap;
  dst.assign(src.begin() + st, src.end());
  std::sort(dst.begin(), dst.end(), by_key<D>);
}

// merge((H - lambda) in) per hash bucket, coefficient 1 and no top-Nd slice: the
// product that spmspvm_bucket_linear (src/functions.cpp:903-966) and
// spmspvm_bucket_res_norm (:1161-1211) build before their bucket-level steps
template <class D>
std::vector<std::vector<Term<D>>> merged_product(const std::vector<Term<D>>& in, double lambda, size_t nb) {
  const int T = g_threads;
  auto bucket_of = [nb](D k) { return (size_t)(hash_det(k) % nb); };
  std::vector<std::vector<Term<D>>> res((size_t)T * nb);
#pragma omp parallel num_threads(T)
  {
    const int tid = omp_get_thread_num();
#pragma omp for schedule(static, 32)
    for (long long i = 0; i < (long long)in.size(); ++i) {
      const D bi = in[i].k;
      const double t = in[i].a;
      off_diag_gen<D>(bi, t, [&](D k, double a) { res[tid + (size_t)T * bucket_of(k)].push_back({k, a}); });
      res[tid + (size_t)T * bucket_of(bi)].push_back({bi, (diag_cal<D>(bi) - lambda) * t});
    }
  }
  std::vector<std::vector<Term<D>>> local(nb);
#pragma omp parallel for schedule(dynamic) num_threads(T)
  for (long long b = 0; b < (long long)nb; ++b) {
    auto& L = local[b];
    for (int j = 0; j < T; ++j) {
      auto& r = res[j + (size_t)T * b];
      L.insert(L.end(), r.begin(), r.end());
    }
    std::sort(L.begin(), L.end(), by_key<D>);
    L.resize(merge_runs(L, L.size()));
  }
  return local;
}

// make_bucket, src/functions.cpp:466-509 (same bucket function as the product)
template <class D> std::vector<std::vector<Term<D>>> bucketed(const std::vector<Term<D>>& v, size_t nb) {
  std::vector<std::vector<Term<D>>> out(nb);
  for (auto& t : v) out[(size_t)(hash_det(t.k) % nb)].push_back(t);
  for (auto& b : out) std::sort(b.begin(), b.end(), by_key<D>);
  return out;
}

// serial cut + top-cap + key sort of the buckets (src/functions.cpp:1007-1086)
template <class D>
void cut_cap_sort(const std::vector<std::vector<Term<D>>>& local, size_t out_cap, std::vector<Term<D>>& out) {
  std::vector<Term<D>> fin;
  for (auto& L : local)
    for (auto& t : L)
      if (std::fabs(t.a) > kCut) fin.push_back(t);
  std::stable_sort(fin.begin(), fin.end(), by_abs<D>);
  size_t s0 = fin.size() < out_cap ? 0 : fin.size() - out_cap;
  out.assign(fin.begin() + s0, fin.end());
  std::sort(out.begin(), out.end(), by_key<D>);
}

// spmspvm_bucket_linear, src/functions.cpp:858-1094: w = (H - lambda) v_cur
// merged; Hij[j] = <w, v_j> for j <= cur before anything is removed (:971-978);
// w -= Hij[cur] v_cur + Hij[cur-1] v_{cur-1} bucket by bucket (:989-997); then
// the cut, the top-cap and the key sort
template <class D>
void spmspv_linear(const std::vector<std::vector<Term<D>>>& basis, unsigned cur, double lambda, size_t out_cap,
                   std::vector<Term<D>>& out, double* hij) {
  out.clear();
  if (basis[cur].empty()) return;  // :880-884 (Hij left as it was)
  for (size_t j = 0; j < basis.size(); ++j) hij[j] = 0.0;
  const size_t nb = (size_t)g_threads * 64;
  auto local = merged_product<D>(basis[cur], lambda, nb);
  std::vector<std::vector<std::vector<Term<D>>>> bb;
  for (auto& v : basis) bb.push_back(bucketed<D>(v, nb));
  for (int j = (int)cur; j >= 0; --j) {
    double s = 0.0;
    for (size_t b = 0; b < nb; ++b) s += dot_sorted(local[b].data(), local[b].size(), bb[j][b].data(), bb[j][b].size());
    hij[j] = s;
  }
  const size_t big = ~(size_t)0;
  for (size_t b = 0; b < nb; ++b) {
    add_two<D>(local[b], big, bb[cur][b], -hij[cur]);
    if (cur > 0) add_two<D>(local[b], big, bb[cur - 1][b], -hij[cur - 1]);
  }
  cut_cap_sort<D>(local, out_cap, out);
}

// spmspvm_bucket_res_norm, src/functions.cpp:1096-1269: w = merge((H - lambda) x)
// - b bucket by bucket; returns |w| before the cut, out = the cut, top-capped w
template <class D>
double res_norm(const std::vector<Term<D>>& x, const std::vector<Term<D>>& bv, double lambda, size_t out_cap,
                std::vector<Term<D>>& out) {
  const size_t nb = (size_t)g_threads * 64;
  auto local = merged_product<D>(x, lambda, nb);
  auto bb = bucketed<D>(bv, nb);
  const size_t big = ~(size_t)0;
  double r = 0.0;
  for (size_t b = 0; b < nb; ++b) {
    add_two<D>(local[b], big, bb[b], -1.0);
    double q = 0.0;
    for (auto& t : local[b]) q += t.a * t.a;
    r += q;
  }
  cut_cap_sort<D>(local, out_cap, out);
  return std::sqrt(r);
}

// ---- word-array <-> determinant conversion -----------------------------------
template <class D> D from_words(const u64* w);
template <> u64 from_words<u64>(const u64* w) { return w[0]; }
template <> u128 from_words<u128>(const u64* w) { return (u128)w[0] | ((u128)w[1] << 64); }
template <class D> void to_words(D d, u64* w);
template <> void to_words<u64>(u64 d, u64* w) { w[0] = d; }
template <> void to_words<u128>(u128 d, u64* w) { w[0] = (u64)d; w[1] = (u64)(d >> 64); }
template <class D> constexpr int words() { return sizeof(D) / 8; }

template <class D> std::vector<Term<D>> load(const u64* k, const double* a, unsigned n) {
  std::vector<Term<D>> v(n);
  for (unsigned i = 0; i < n; ++i) v[i] = {from_words<D>(k + (size_t)i * words<D>()), a[i]};
  return v;
}
template <class D> void store(const std::vector<Term<D>>& v, u64* k, double* a, unsigned* n) {
  for (size_t i = 0; i < v.size(); ++i) {
    to_words<D>(v[i].k, k + i * words<D>());
    a[i] = v[i].a;
  }
  *n = (unsigned)v.size();
}

int setup(const char* path, unsigned norb, unsigned ne, unsigned nd, unsigned nthread) {
  H = Ham();
  H.N = (int)norb;
  H.ne = (int)ne;
  H.OO.assign((size_t)norb * norb, {});
  H.OO_c.assign((size_t)norb * norb, {});
  H.O.assign(norb, {});
  H.O_c.assign(norb, {});
  g_Nd = nd;
  g_threads = nthread ? (int)nthread : omp_get_max_threads();
  return read_elements(path) ? 0 : -1;
}

}  // namespace

#define PORT_API(W, D)                                                                                           \
  extern "C" int port##W##_setup(const char* p, unsigned norb, unsigned ne, unsigned nd, unsigned, unsigned nt, \
                                 unsigned) {                                                                     \
    return setup(p, norb, ne, nd, nt);                                                                           \
  }                                                                                                              \
  extern "C" void port##W##_set_nd(unsigned nd) { g_Nd = nd; }                                                   \
  extern "C" void port##W##_set_cut(double cut) { kCut = cut; }                                                  \
  extern "C" void port##W##_spmspv(const u64* ik, const double* ia, unsigned il, unsigned, unsigned ocap,      \
                                   double lam, double coeff, u64* ok, double* oa, unsigned* ol, double* dg) {   \
    std::vector<Term<D>> out;                                                                                    \
    spmspv<D>(load<D>(ik, ia, il), ocap, lam, coeff, out, dg);                                                   \
    store<D>(out, ok, oa, ol);                                                                                   \
  }                                                                                                              \
  extern "C" void port##W##_spmspv_linear(const u64* bk, const double* ba, const unsigned* blen, unsigned nbv,   \
                                          unsigned cur, double lam, unsigned ocap, u64* ok, double* oa,         \
                                          unsigned* ol, double* hij) {                                          \
    std::vector<std::vector<Term<D>>> basis(nbv);                                                                \
    size_t off = 0;                                                                                              \
    for (unsigned j = 0; j < nbv; ++j) {                                                                         \
      basis[j] = load<D>(bk + off * words<D>(), ba + off, blen[j]);                                              \
      off += blen[j];                                                                                            \
    }                                                                                                            \
    std::vector<Term<D>> out;                                                                                    \
    spmspv_linear<D>(basis, cur, lam, ocap, out, hij);                                                           \
    store<D>(out, ok, oa, ol);                                                                                   \
  }                                                                                                              \
  extern "C" double port##W##_res_norm(const u64* xk, const double* xa, unsigned xl, const u64* bk,             \
                                       const double* ba, unsigned bl, double lam, unsigned ocap, u64* ok,        \
                                       double* oa, unsigned* ol) {                                               \
    std::vector<Term<D>> out;                                                                                    \
    double r = res_norm<D>(load<D>(xk, xa, xl), load<D>(bk, ba, bl), lam, ocap, out);                            \
    store<D>(out, ok, oa, ol);                                                                                   \
    return r;                                                                                                    \
  }                                                                                                              \
  extern "C" double port##W##_energy(const u64* k, const double* a, unsigned n) { return energy<D>(load<D>(k, a, n)); } \
  extern "C" double port##W##_dot(const u64* k1, const double* a1, unsigned l1, const u64* k2, const double* a2, \
                                  unsigned l2) {                                                                 \
    auto x = load<D>(k1, a1, l1);                                                                                \
    auto y = load<D>(k2, a2, l2);                                                                                \
    return dot_sorted<D>(x.data(), x.size(), y.data(), y.size());                                                \
  }                                                                                                              \
  extern "C" double port##W##_norm(const u64*, const double* a, unsigned n) {                                   \
    double s = 0;                                                                                                \
    for (unsigned i = 0; i < n; ++i) s += a[i] * a[i];                                                           \
    return std::sqrt(s);                                                                                         \
  }                                                                                                              \
  extern "C" void port##W##_add_two(const u64* vk, const double* va, unsigned vl, unsigned vcap, const u64* wk, \
                                    const double* wa, unsigned wl, double a, u64* ok, double* oa, unsigned* ol) { \
    auto v = load<D>(vk, va, vl);                                                                                \
    add_two<D>(v, vcap, load<D>(wk, wa, wl), a);                                                                 \
    store<D>(v, ok, oa, ol);                                                                                     \
  }                                                                                                              \
  extern "C" void port##W##_add_three(const u64* xk, const double* xa, unsigned xl, const u64* yk,               \
                                      const double* ya, unsigned yl, const u64* zk, const double* za,            \
                                      unsigned zl, double a, double b, double c, u64* ok, double* oa,            \
                                      unsigned* ol) {                                                            \
    std::vector<Term<D>> v;                                                                                      \
    add_three<D>(v, load<D>(xk, xa, xl), load<D>(yk, ya, yl), load<D>(zk, za, zl), a, b, c);                     \
    store<D>(v, ok, oa, ol);                                                                                     \
  }                                                                                                              \
  extern "C" void port##W##_shrink_from(const u64* sk, const double* sa, unsigned sl, unsigned dcap, u64* ok,   \
                                        double* oa, unsigned* ol) {                                              \
    std::vector<Term<D>> d;                                                                                      \
    shrink_from<D>(d, dcap, load<D>(sk, sa, sl));                                                                \
    store<D>(d, ok, oa, ol);                                                                                     \
  }                                                                                                              \
  extern "C" unsigned port##W##_sort_merge(u64* k, double* a, unsigned n) {                                     \
    auto v = load<D>(k, a, n);                                                                                   \
    std::stable_sort(v.begin(), v.end(), by_key<D>);                                                             \
    v.resize(merge_runs(v, v.size()));                                                                           \
    unsigned m;                                                                                                  \
    store<D>(v, k, a, &m);                                                                                       \
    return m;                                                                                                    \
  }

PORT_API(64, u64)
PORT_API(128, u128)

extern "C" double port64_diag(u64 d) { return diag_cal<u64>(d); }
extern "C" double port128_diag(u64 lo, u64 hi) { return diag_cal<u128>((u128)lo | ((u128)hi << 64)); }

extern "C" unsigned port64_offdiag(u64 d, u64* k, double* a, unsigned cap) {
  unsigned n = 0;
  off_diag_gen<u64>(d, 1.0, [&](u64 kk, double aa) {
    if (n < cap) { k[n] = kk; a[n] = aa; }
    ++n;
  });
  return n;
}
extern "C" unsigned port128_offdiag(u64 lo, u64 hi, u64* k, double* a, unsigned cap) {
  unsigned n = 0;
  off_diag_gen<u128>((u128)lo | ((u128)hi << 64), 1.0, [&](u128 kk, double aa) {
    if (n < cap) { k[2 * n] = (u64)kk; k[2 * n + 1] = (u64)(kk >> 64); a[n] = aa; }
    ++n;
  });
  return n;
}
