// Host-side set-up: wavenumber tables and integrating factor (defk.f90),
// forced-mode enumeration (iniforcing_3d3c.f90 / iniforcing_2d2c.f90), the
// reference RNG and forcing draws (forcing_3d3c.f90 / forcing_2d2c.f90),
// the initial noise (trunc.f90:75-93), params.dat parsing
// (inieuler.f90:14-20), seed and field files (main.f90:37-45, read.f90,
// write.f90).  No CUDA here: everything in this file runs without a GPU.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <thread>
#include <unordered_set>
#include <vector>

#include "gt_internal.h"

namespace gt {

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

double emk_value(const gt_params& p, double k2) {
  // defk.f90:61-65: scra = nu fk2**alpnu + mu fk2**alpmu (fk2 /= 0);
  // emk = dexp(-0.5*dt*scra), with the REAL*4 literal 0.5 (exact).
  if (k2 == 0.0) return 1.0;
  double scra = p.nu * std::pow(k2, p.alpnu) + p.mu * std::pow(k2, p.alpmu);
  return std::exp((-0.5 * p.dt) * scra);
}

int build_tables(const gt_params& p, HostTables& t) {
  const int nx = p.nx, ny = p.ny, nz = p.nz, nh = nx / 2 + 1;
  t.nx = nx; t.ny = ny; t.nz = nz; t.nh = nh;
  // defk.f90:13-21
  t.jc.assign(ny, 0); t.kc.assign(nz, 0);
  for (int j = 1; j < ny; ++j) t.jc[j] = ny - j;
  for (int k = 1; k < nz; ++k) t.kc[k] = nz - k;
  // defk.f90:24-43
  const double dkx = 2.0 * kPiRef / p.xlx, dky = 2.0 * kPiRef / p.xly, dkz = 2.0 * kPiRef / p.xlz;
  t.fkx.resize(nh); t.fky.resize(ny); t.fkz.resize(nz);
  for (int i = 0; i < nh; ++i) t.fkx[i] = (double)i * dkx;
  for (int j = 0; j < ny; ++j) t.fky[j] = (j <= ny / 2 ? (double)j : (double)(j - ny)) * dky;
  for (int k = 0; k < nz; ++k) t.fkz[k] = (k <= nz / 2 ? (double)k : (double)(k - nz)) * dkz;
  // defk.f90:46-54
  t.fkxs.resize(nh); t.fkys.resize(ny); t.fkzs.resize(nz);
  for (int i = 0; i < nh; ++i) t.fkxs[i] = t.fkx[i] * t.fkx[i];
  for (int j = 0; j < ny; ++j) t.fkys[j] = t.fky[j] * t.fky[j];
  for (int k = 0; k < nz; ++k) t.fkzs[k] = t.fkz[k] * t.fkz[k];
  // defk.f90:88-91
  t.fkxsmax = t.fkxs[nh - 1];
  t.fkysmax = t.fkys[ny / 2];
  t.fkzsmax = t.fkzs[nz / 2];
  t.rtrunc2 = p.rtrunc * p.rtrunc;

  // Integrating factor.  With integer wavenumbers (the 2 pi box) fk2 is an
  // exact integer and emk depends on it alone: keep one value per integer k2.
  bool integer = true;
  auto chk = [&](const std::vector<double>& v) {
    for (double x : v) if (x != std::floor(x) || std::fabs(x) > 4096.0) integer = false;
  };
  chk(t.fkx); chk(t.fky); chk(t.fkz);
  if (integer) {
    double k2max = t.fkxs[nh - 1];
    double ym = 0, zm = 0;
    for (double v : t.fkys) ym = std::max(ym, v);
    for (double v : t.fkzs) zm = std::max(zm, v);
    k2max = (k2max + ym) + zm;
    t.emk_by_k2 = true;
    t.emk_k2.resize((size_t)k2max + 1);
    for (size_t m = 0; m <= (size_t)k2max; ++m) t.emk_k2[m] = emk_value(p, (double)m);
    t.emk_full.clear();
  } else {
    t.emk_by_k2 = false;
    t.emk_full.resize((size_t)nz * ny * nh);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nh; ++i) {
          double fk2 = (t.fkxs[i] + t.fkys[j]) + t.fkzs[k];   // defk.f90:61
          t.emk_full[((size_t)k * ny + j) * nh + i] = emk_value(p, fk2);
        }
  }

  // trunc.f90:14-17: zero where ((kz2/kz2max + ky2/ky2max) + kx2/kx2max) > rtrunc^2.
  // The sum is non-decreasing in kx2 >= 0, so the kept modes of a row form a
  // prefix ix < xcut.
  t.xcut.assign((size_t)nz * ny, nh);
  if (p.truncate == 1) {
    for (int k = 0; k < nz; ++k) {
      const double k3 = t.fkzs[k] / t.fkzsmax;
      for (int j = 0; j < ny; ++j) {
        const double k2 = k3 + t.fkys[j] / t.fkysmax;
        int cut = nh;
        for (int i = 0; i < nh; ++i) {
          const double k1 = k2 + t.fkxs[i] / t.fkxsmax;
          if (k1 > t.rtrunc2) { cut = i; break; }
        }
        t.xcut[(size_t)k * ny + j] = cut;
      }
    }
  }

  // Forced modes (iniforcing_3d3c.f90:22-184 / iniforcing_2d2c.f90:17-73).
  t.fix.clear(); t.fiy.clear(); t.fiz.clear(); t.ff.clear();
  t.inpe = 0; t.inpz = 0;
  if (p.forcing == GT_FORCING_NONE) return GT_OK;
  const int nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
  std::vector<double> k2list;
  bool overflow = false;
  auto visit = [&](int i, int j, int k, bool inline_inputs) {
    if (overflow) return;
    const double k2 = (t.fkxs[i] + t.fkys[j]) + t.fkzs[k];
    const double k2n = (t.fkxs[i] / t.fkxsmax + t.fkys[j] / t.fkysmax) + t.fkzs[k] / t.fkzsmax;
    if (!(k2n <= t.rtrunc2)) return;
    if (!((k2 <= p.k2f * p.k2f) && (k2 > p.k1f * p.k1f))) return;
    if ((int)t.fix.size() + 1 > GT_NFORC) { overflow = true; return; }
    const double kk = std::sqrt(k2);
    const double f = 1.0 / kk;
    t.fix.push_back(i); t.fiy.push_back(j); t.fiz.push_back(k); t.ff.push_back(f);
    k2list.push_back(k2);
    if (inline_inputs) {  // iniforcing_3d3c.f90:38-39
      const double a = p.famp * f;
      t.inpz = t.inpz + k2 * k2 * (a * a);
      t.inpe = t.inpe + k2 * (a * a);
    }
  };
  if (p.forcing == GT_FORCING_3D3C) {
    for (int k = 1; k < nz2; ++k) visit(0, 0, k, true);                       // :22-43
    for (int j = 1; j < ny2; ++j) for (int k = 0; k < nz; ++k) visit(0, j, k, true);   // :45-66
    for (int k = 1; k < nz2; ++k) visit(0, ny2, k, true);                     // :68-88
    for (int i = 1; i < nx2; ++i)                                             // :91-114
      for (int j = 0; j < ny; ++j) for (int k = 0; k < nz; ++k) visit(i, j, k, true);
    for (int k = 1; k < nz2; ++k) visit(nx2, 0, k, true);                     // :117-139
    for (int j = 1; j < ny2; ++j) for (int k = 0; k < nz; ++k) visit(nx2, j, k, true); // :141-162
    for (int k = 1; k < nz2; ++k) visit(nx2, ny2, k, true);                   // :164-184
  } else {
    for (int j = 1; j < ny2; ++j) visit(0, j, 0, false);                      // :17-32
    for (int i = 1; i < nx2; ++i) for (int j = 0; j < ny; ++j) visit(i, j, 0, false);  // :34-50
    for (int j = 1; j < ny2; ++j) visit(nx2, j, 0, false);                    // :52-67
    for (size_t m = 0; m < k2list.size(); ++m) {                              // :69-73
      const double a = p.famp * t.ff[m];
      t.inpe = t.inpe + k2list[m] * (a * a);
      t.inpz = t.inpz + k2list[m] * k2list[m] * (a * a);
    }
  }
  if (overflow) return GT_ENFORC;
  return GT_OK;
}

float rann(int32_t& irand) {
  // irand = iand(69069*irand + 1, '7FFFFFFF'X) in 32-bit wraparound
  // arithmetic; rann = dble(irand)/dble(mask), returned as REAL*4.
  uint32_t x = (uint32_t)irand;
  x = x * (uint32_t)kLcgMul + 1u;
  irand = (int32_t)(x & (uint32_t)kLcgMask);
  return (float)((double)irand / (double)kLcgMask);
}

// The LCG step x -> (69069 x + 1) mod 2^31 applied m times is the affine map
// x -> (am x + cm) mod 2^31; composing maps by squaring gives (am, cm) in
// log2 m steps, so that threads can start at any position of the stream.
static void lcg_jump(uint64_t m, uint32_t& am, uint32_t& cm) {
  uint32_t a = 1u, c = 0u;                          // accumulated map
  uint32_t pa = (uint32_t)kLcgMul, pc = 1u;         // the map of 2^bit steps
  while (m) {
    if (m & 1u) {                                   // accumulated after (pa, pc)
      c = (pa * c + pc) & (uint32_t)kLcgMask;
      a = (pa * a) & (uint32_t)kLcgMask;
    }
    pc = (pa * pc + pc) & (uint32_t)kLcgMask;
    pa = (pa * pa) & (uint32_t)kLcgMask;
    m >>= 1;
  }
  am = a;
  cm = c;
}

void init_noise(const gt_params& p, int32_t& seed, double* ux, double* uy, double* uz) {
  // trunc.f90:75-93: for k, j, i: b{x,y,z}(i,j,k) += sdt*(rann(seed)-0.5),
  // the three components of a point drawn in turn; rann - 0.5 is REAL*4
  // arithmetic, promoted to REAL*8 by the product with sdt = sqrt(dt)
  // (inieuler.f90:67).  The arrays start at zero (inieuler.f90:79-81), so the
  // result is the noise itself.
  const double sdt = std::sqrt(p.dt);
  const size_t npts = (size_t)p.nx * p.ny * p.nz;
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > 64) nt = 64;
  if (npts < (size_t)nt * 65536) nt = 1;
  const uint32_t x0 = (uint32_t)seed & (uint32_t)kLcgMask;
  auto work = [&](size_t p0, size_t p1) {
    uint32_t am, cm;
    lcg_jump(3ull * p0, am, cm);
    int32_t irand = (int32_t)((am * x0 + cm) & (uint32_t)kLcgMask);
    for (size_t q = p0; q < p1; ++q) {
      ux[q] = sdt * (double)(rann(irand) - 0.5f);
      uy[q] = sdt * (double)(rann(irand) - 0.5f);
      uz[q] = sdt * (double)(rann(irand) - 0.5f);
    }
  };
  std::vector<std::thread> pool;
  const size_t chunk = (npts + nt - 1) / nt;
  for (unsigned i = 1; i < nt; ++i) {
    const size_t p0 = i * chunk, p1 = std::min(npts, p0 + chunk);
    if (p0 < p1) pool.emplace_back(work, p0, p1);
  }
  work(0, std::min(npts, chunk));
  for (auto& th : pool) th.join();
  uint32_t am, cm;
  lcg_jump(3ull * npts, am, cm);
  seed = (int32_t)((am * x0 + cm) & (uint32_t)kLcgMask);
}

void draw_forcing(const gt_params& p, const HostTables& t, int32_t& seed,
                  std::vector<ForceEntry>& out) {
  const double sf = std::sqrt(p.dt) * p.famp;  // sdt*famp (inieuler.f90:67, forcing_3d3c.f90:35)
  const int nx2 = p.nx / 2;
  const size_t nf = t.fix.size();
  for (size_t ik = 0; ik < nf; ++ik) {
    const int i = t.fix[ik], j = t.fiy[ik], k = t.fiz[ik];
    if (p.forcing == GT_FORCING_3D3C) {
      double te = kPi2_3d3c * (double)rann(seed);                   // :34
      const double er0 = sf * std::cos(te), ei0 = sf * std::sin(te);   // :35
      te = kPi2_3d3c * (double)rann(seed);                          // :38
      const double cte = std::cos(te), ste = std::sin(te);          // :39-40
      const double er = er0 * t.ff[ik], ei = ei0 * t.ff[ik];       // :42 effek = effe*ff
      if (i == 0 && j == 0) {                                       // :45-50
        ForceEntry a{k, j, i, 3, {er * cte, ei * cte, er * ste, ei * ste, 0, 0}};
        ForceEntry c{t.kc[k], t.jc[j], i, 3, {er * cte, -ei * cte, er * ste, -ei * ste, 0, 0}};
        out.push_back(a);
        out.push_back(c);
      } else {                                                      // :52-68
        double k2 = t.fkxs[i] + t.fkys[j];
        const double kxy = std::sqrt(k2);
        k2 = k2 + t.fkzs[k];
        const double kk = std::sqrt(k2);
        const double c1 = t.fkz[k] / kk, s1 = kxy / kk;
        const double c2 = t.fkx[i] / kxy, s2 = t.fky[j] / kxy;
        const double fx = cte * c2 * c1 - ste * s2;
        const double fy = cte * s2 * c1 + ste * c2;
        ForceEntry a{k, j, i, 7,
                     {er * fx, ei * fx, er * fy, ei * fy, -((er * cte) * s1), -((ei * cte) * s1)}};
        out.push_back(a);
        if (i == 0 || i == nx2) {
          ForceEntry c{t.kc[k], t.jc[j], i, 7,
                       {er * fx, -ei * fx, er * fy, -ei * fy, -((er * cte) * s1),
                        -((-ei * cte) * s1)}};
          out.push_back(c);
        }
      }
    } else if (p.forcing == GT_FORCING_2D2C) {
      const double te = kPi2_2d2c * (double)rann(seed);             // forcing_2d2c.f90:33
      const double er0 = sf * std::cos(te), ei0 = sf * std::sin(te);   // :34
      const double er = er0 * t.ff[ik], ei = ei0 * t.ff[ik];       // :35
      out.push_back(ForceEntry{k, j, i, 4, {0, 0, 0, 0, er, ei}});   // :37
      if (i == 0 || i == nx2)                                        // :38-41
        out.push_back(ForceEntry{t.kc[k], t.jc[j], i, 4, {0, 0, 0, 0, er, -ei}});
    }
  }
}

bool entries_unique(const ForceEntry* e, size_t n) {
  std::unordered_set<uint64_t> seen;
  seen.reserve(n * 2);
  for (size_t i = 0; i < n; ++i) {
    uint64_t key = ((uint64_t)(uint32_t)e[i].z << 42) | ((uint64_t)(uint32_t)e[i].y << 21) |
                   (uint64_t)(uint32_t)e[i].x;
    if (!seen.insert(key).second) return false;
  }
  return true;
}

}  // namespace gt

using namespace gt;

extern "C" {

int gt_params_default(gt_params* p) {
  if (!p) return GT_EINVAL;
  std::memset(p, 0, sizeof(*p));
  p->nx = p->ny = p->nz = 64;
  p->xlx = p->xly = p->xlz = 2.0 * kPiRef;
  p->nu = 2e-3; p->alpnu = 1.0; p->mu = 0.0; p->alpmu = 0.0;
  p->dt = 5e-3; p->omega = 5.0;
  p->rtrunc = 0.6666666666666666667; p->truncate = 1;
  p->famp = 0.0; p->k1f = 1.999; p->k2f = 3.0;
  p->forcing = GT_FORCING_3D3C;
  p->dt2_mode = GT_DT2_RK2;
  p->precision = GT_PREC_FP64;
  p->device = 0;
  return GT_OK;
}

int gt_params_validate(const gt_params* p) {
  if (!p) return GT_EINVAL;
  const int dims[3] = {p->nx, p->ny, p->nz};
  for (int d : dims)
    if (!is_pow2(d) || d < 8 || d > 1024) return GT_EINVAL;
  if (!(p->xlx > 0) || !(p->xly > 0) || !(p->xlz > 0)) return GT_EINVAL;
  if (!std::isfinite(p->dt) || !(p->dt > 0)) return GT_EINVAL;
  if (!std::isfinite(p->nu) || !std::isfinite(p->mu) || !std::isfinite(p->alpnu) ||
      !std::isfinite(p->alpmu) || !std::isfinite(p->omega) || !std::isfinite(p->famp))
    return GT_EINVAL;
  if (!(p->rtrunc > 0) || (p->truncate != 0 && p->truncate != 1)) return GT_EINVAL;
  if (p->forcing < GT_FORCING_NONE || p->forcing > GT_FORCING_2D2C) return GT_EINVAL;
  if (p->dt2_mode != GT_DT2_AS_BUILT && p->dt2_mode != GT_DT2_RK2) return GT_EINVAL;
  if (p->precision != GT_PREC_FP64 && p->precision != GT_PREC_MIXED) return GT_EINVAL;
  if (p->device < 0) return GT_EINVAL;
  return GT_OK;
}

// Fortran list-directed reading of one "read(9,*) a, b, ..." statement:
// takes as many whitespace/comma separated values as requested, continuing
// on following lines, then discards the rest of the last line.  The 'd'
// exponent letter is accepted.
static bool read_values(std::istream& in, int n, std::vector<std::string>& out) {
  out.clear();
  std::string line;
  while ((int)out.size() < n) {
    if (!std::getline(in, line)) return false;
    for (char& ch : line) if (ch == ',' || ch == '\t') ch = ' ';
    std::istringstream ls(line);
    std::string tok;
    while ((int)out.size() < n && (ls >> tok)) {
      for (char& ch : tok) if (ch == 'd' || ch == 'D') ch = 'e';
      out.push_back(tok);
    }
  }
  return true;
}

static bool to_double(const std::string& s, double& v) {
  char* end = nullptr;
  v = std::strtod(s.c_str(), &end);
  return end && *end == '\0' && end != s.c_str();
}

// A list-directed integer item: an optional sign and decimal digits only (a
// Fortran integer read rejects "3.0" and "1e3"), within the int32 range.
static bool to_int(const std::string& s, int32_t& v) {
  size_t i = 0;
  bool neg = false;
  if (i < s.size() && (s[i] == '+' || s[i] == '-')) neg = (s[i++] == '-');
  if (i == s.size()) return false;
  int64_t acc = 0;
  for (; i < s.size(); ++i) {
    if (s[i] < '0' || s[i] > '9') return false;
    acc = acc * 10 + (s[i] - '0');
    if (acc > (int64_t)INT32_MAX + 1) return false;   // stops before int64 overflow
  }
  if (neg) acc = -acc;
  if (acc < (int64_t)INT32_MIN || acc > (int64_t)INT32_MAX) return false;
  v = (int32_t)acc;
  return true;
}

int gt_params_read(const char* path, gt_params* p) {
  if (!path || !p) return GT_EINVAL;
  std::ifstream in(path);
  if (!in) return GT_EIO;
  std::vector<std::string> v;
  double d[4];
  int32_t iv[3];
  // inieuler.f90:14 xlx,xly,xlz
  if (!read_values(in, 3, v)) return GT_EIO;
  for (int i = 0; i < 3; ++i) if (!to_double(v[i], d[i])) return GT_EIO;
  gt_params q = *p;
  q.xlx = d[0]; q.xly = d[1]; q.xlz = d[2];
  // :15 nu,alpnu,mu,alpmu
  if (!read_values(in, 4, v)) return GT_EIO;
  for (int i = 0; i < 4; ++i) if (!to_double(v[i], d[i])) return GT_EIO;
  q.nu = d[0]; q.alpnu = d[1]; q.mu = d[2]; q.alpmu = d[3];
  // :16 dt,omega
  if (!read_values(in, 2, v)) return GT_EIO;
  for (int i = 0; i < 2; ++i) if (!to_double(v[i], d[i])) return GT_EIO;
  q.dt = d[0]; q.omega = d[1];
  // :17 npas,iout,imix (run control; kept by the driver, not by the step)
  if (!read_values(in, 3, v)) return GT_EIO;
  for (int i = 0; i < 3; ++i) if (!to_int(v[i], iv[i])) return GT_EIO;
  // :18 rtrunc,truncate
  if (!read_values(in, 2, v)) return GT_EIO;
  if (!to_double(v[0], d[0]) || !to_int(v[1], iv[0])) return GT_EIO;
  q.rtrunc = d[0]; q.truncate = iv[0];
  // :19 famp,k1f,k2f
  if (!read_values(in, 3, v)) return GT_EIO;
  for (int i = 0; i < 3; ++i) if (!to_double(v[i], d[i])) return GT_EIO;
  q.famp = d[0]; q.k1f = d[1]; q.k2f = d[2];
  *p = q;
  return GT_OK;
}

int gt_memory_estimate(const gt_params* p, size_t* bytes) {
  if (!p || !bytes) return GT_EINVAL;
  int rc = gt_params_validate(p);
  if (rc) return rc;
  const size_t esz = p->precision == GT_PREC_FP64 ? 16 : 8;
  const size_t align = 128 / esz;
  const size_t nh = (size_t)p->nx / 2 + 1;
  const size_t nhp = (nh + align - 1) / align * align;
  const size_t field = nhp * p->ny * p->nz * esz;
  // 3 state + 3 stage + 6 work fields, plus tables, staging and partials
  size_t total = 12 * field;
  total += (size_t)p->nz * p->ny * 4 + (size_t)(3 * 1024 + 1024 * 1024 * 3) * 8;
  *bytes = total;
  return GT_OK;
}

namespace {
std::atomic<uint64_t> g_memory_budget{0};
}  // namespace

int gt_set_memory_budget(uint64_t bytes) {
  g_memory_budget.store(bytes);
  return GT_OK;
}

int gt_get_memory_budget(uint64_t* bytes) {
  if (!bytes) return GT_EINVAL;
  *bytes = g_memory_budget.load();
  return GT_OK;
}

int gt_rann(int32_t* irand, int32_t n, float* out) {
  if (!irand || n < 0 || (n > 0 && !out)) return GT_EINVAL;
  for (int32_t i = 0; i < n; ++i) out[i] = rann(*irand);
  return GT_OK;
}

int gt_init_noise(const gt_params* p, int32_t* seed, double* ux, double* uy, double* uz) {
  if (!p || !seed || !ux || !uy || !uz) return GT_EINVAL;
  const int rc = gt_params_validate(p);
  if (rc) return rc;
  gt::init_noise(*p, *seed, ux, uy, uz);
  return GT_OK;
}

int gt_forced_modes(const gt_params* p, int32_t* nf, int32_t* ix, int32_t* iy, int32_t* iz,
                    double* ff, double* inpe, double* inpz) {
  if (!p) return GT_EINVAL;
  int rc = gt_params_validate(p);
  if (rc) return rc;
  HostTables t;
  rc = build_tables(*p, t);
  if (rc) return rc;
  const size_t n = t.fix.size();
  if (nf) *nf = (int32_t)n;
  for (size_t m = 0; m < n; ++m) {
    if (ix) ix[m] = t.fix[m];
    if (iy) iy[m] = t.fiy[m];
    if (iz) iz[m] = t.fiz[m];
    if (ff) ff[m] = t.ff[m];
  }
  if (inpe) *inpe = t.inpe;
  if (inpz) *inpz = t.inpz;
  return GT_OK;
}

int gt_forcing_increments(const gt_params* p, int32_t* seed, int32_t cap, int32_t* n,
                          int32_t* ix, int32_t* iy, int32_t* iz, double* dF) {
  if (!p || !seed || !n || cap < 0) return GT_EINVAL;
  int rc = gt_params_validate(p);
  if (rc) return rc;
  HostTables t;
  rc = build_tables(*p, t);
  if (rc) return rc;
  std::vector<ForceEntry> e;
  int32_t s = *seed;
  draw_forcing(*p, t, s, e);
  if ((int64_t)e.size() > cap) return GT_EINVAL;
  if (e.size() > 0 && (!ix || !iy || !iz || !dF)) return GT_EINVAL;
  for (size_t m = 0; m < e.size(); ++m) {
    ix[m] = e[m].x;
    iy[m] = e[m].y;
    iz[m] = e[m].z;
    for (int q = 0; q < 6; ++q) dF[m * 6 + q] = (e[m].mask & (1 << (q / 2))) ? e[m].inc[q] : 0.0;
  }
  *n = (int32_t)e.size();
  *seed = s;
  return GT_OK;
}

int gt_seed_read(const char* path, int32_t* seed) {
  if (!path || !seed) return GT_EINVAL;
  std::ifstream in(path);
  if (!in) return GT_EIO;
  std::vector<std::string> v;
  if (!read_values(in, 1, v)) return GT_EIO;
  int32_t s;
  if (!to_int(v[0], s)) return GT_EIO;
  *seed = s;
  return GT_OK;
}

int gt_seed_write(const char* path, int32_t seed) {
  if (!path) return GT_EINVAL;
  FILE* f = std::fopen(path, "w");
  if (!f) return GT_EIO;
  int ok = std::fprintf(f, " %12d\n", seed) > 0;   // list-directed integer write
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GT_OK : GT_EIO;
}

int gt_frame_read(const char* path, int32_t* ifr, double* t) {
  // main.f90:37-39: read(1,*) ifr, t
  if (!path || !ifr || !t) return GT_EINVAL;
  std::ifstream in(path);
  if (!in) return GT_EIO;
  std::vector<std::string> v;
  if (!read_values(in, 2, v)) return GT_EIO;
  int32_t f;
  double tt;
  if (!to_int(v[0], f) || !to_double(v[1], tt)) return GT_EIO;
  *ifr = f;
  *t = tt;
  return GT_OK;
}

int gt_frame_write(const char* path, int32_t ifr, double t) {
  // main.f90:213-215: write(1,*) ifr, t (list-directed; 17 significant digits
  // read back exactly)
  if (!path) return GT_EINVAL;
  FILE* f = std::fopen(path, "w");
  if (!f) return GT_EIO;
  int ok = std::fprintf(f, " %12d %25.17E\n", ifr, t) > 0;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GT_OK : GT_EIO;
}

// Fortran unformatted sequential records: a 4-byte length marker before and
// after the data.  Records longer than 2^31-1 bytes are split into
// sub-records whose leading marker is negative while more follow (the
// gfortran convention); both forms are accepted on input.
int gt_field_read_f32(const char* path, int32_t nx, int32_t ny, int32_t nz, float* out) {
  if (!path || !out || nx <= 0 || ny <= 0 || nz <= 0) return GT_EINVAL;
  FILE* f = std::fopen(path, "rb");
  if (!f) return GT_EIO;
  const size_t want = (size_t)nx * ny * nz * sizeof(float);
  size_t got = 0;
  char* dst = reinterpret_cast<char*>(out);
  while (got < want) {
    int32_t head, tail;
    if (std::fread(&head, 4, 1, f) != 1) { std::fclose(f); return GT_EIO; }
    const size_t len = (size_t)(head < 0 ? -(int64_t)head : head);
    if (len > want - got) { std::fclose(f); return GT_EIO; }
    if (std::fread(dst + got, 1, len, f) != len) { std::fclose(f); return GT_EIO; }
    if (std::fread(&tail, 4, 1, f) != 1) { std::fclose(f); return GT_EIO; }
    if ((size_t)(tail < 0 ? -(int64_t)tail : tail) != len) { std::fclose(f); return GT_EIO; }
    got += len;
    if (head >= 0 && got < want) { std::fclose(f); return GT_EIO; }  // short record
  }
  std::fclose(f);
  return GT_OK;
}

int gt_field_write_f32(const char* path, int32_t nx, int32_t ny, int32_t nz, const float* in) {
  if (!path || !in || nx <= 0 || ny <= 0 || nz <= 0) return GT_EINVAL;
  FILE* f = std::fopen(path, "wb");
  if (!f) return GT_EIO;
  const size_t total = (size_t)nx * ny * nz * sizeof(float);
  const size_t maxrec = 0x7FFFFFFFu - 7u;   // largest multiple of 8 below 2^31
  size_t done = 0;
  const char* src = reinterpret_cast<const char*>(in);
  bool ok = true;
  do {
    const size_t len = std::min(maxrec, total - done);
    const bool more = done + len < total;
    const int32_t head = more ? -(int32_t)len : (int32_t)len;
    const int32_t tail = (done > 0) ? -(int32_t)len : (int32_t)len;
    ok = ok && std::fwrite(&head, 4, 1, f) == 1;
    ok = ok && std::fwrite(src + done, 1, len, f) == len;
    ok = ok && std::fwrite(&tail, 4, 1, f) == 1;
    done += len;
  } while (ok && done < total);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GT_OK : GT_EIO;
}

const char* gt_strerror(int code) {
  switch (code) {
    case GT_OK: return "ok";
    case GT_EINVAL: return "invalid argument or parameter";
    case GT_ENOMEM: return "out of memory (device or host)";
    case GT_ECUDA: return "CUDA runtime error (no usable GPU or a failed launch)";
    case GT_ENFORC: return "NFORC too small: more forced modes than 2048";
    case GT_ENONFINITE: return "state holds NaN or Inf";
    case GT_EIO: return "file missing, unreadable or malformed";
    case GT_ETIMEOUT: return "a bounded device wait timed out";
    default: return "unknown status";
  }
}

}  // extern "C"
