// Host side of the GB300 DMD path (see include/dmd_host.h): DMD's input readers and set-up restated
// in C++, and DMD's time loop driving the GPU ABI. Compiled with -ffp-contract=off so that every
// set-up value rounds as the reference's scalar code does.
#include "dmd_host.h"

#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace {

// comm/Units.h
const double kEV = 1 / 27.21138505;
const double kJoule = 1 / 4.35974434e-18;
const double kAngstrom = 1 / 0.5291772;
const double kMeter = 1e10 * kAngstrom;
const double kKg = 1. / 9.10938291e-31;
const double kNewton = kJoule / kMeter;
const double kSec = sqrt((kKg * kMeter) / kNewton);
const double kFs = kSec * 1.0e-15;
const double kTesla2au = 1. / 2.3505175675871e5;
const double kBohr2cm = 5.291772109038e-9;

thread_local std::string g_err;

int err(int code, const std::string& m) {
  g_err = m;
  return code;
}

bool exists(const std::string& name) {
  struct stat b;
  return stat(name.c_str(), &b) == 0;
}
bool is_dir(const std::string& name) {
  struct stat b;
  return stat(name.c_str(), &b) == 0 && S_ISDIR(b.st_mode);
}

std::string trim(std::string s) {
  s.erase(0, s.find_first_not_of(" "));
  size_t p = s.find_last_not_of(" \n\r\t");
  return p == std::string::npos ? std::string() : s.erase(p + 1);
}

// parameters::map_input (parameters.cpp:591-623), including its key = substr(0, '=' - 1) convention
std::map<std::string, std::string> map_input(std::istream& fin) {
  std::map<std::string, std::string> param;
  bool b_join = false, b_joined = false, b_will_join = false;
  std::string last_key;
  for (std::string line; std::getline(fin, line);) {
    b_will_join = false;
    b_joined = false;
    std::string line2 = trim(line);
    if (!line.empty() && line[0] == '#') continue;
    if (!line2.empty() && line2[line2.length() - 1] == '\\') {
      b_will_join = true;
      line2[line2.length() - 1] = ' ';
    }
    if (b_join) {
      param[last_key] += " " + line2;
      b_joined = true;
    }
    b_join = b_will_join;
    if (!b_joined) {
      size_t eq = line2.find('=');
      if (eq == std::string::npos) continue;
      last_key = trim(line2.substr(0, eq == 0 ? 0 : eq - 1));
      param[last_key] = trim(line2.substr(eq + 1, line2.length() - eq - 1));
    }
  }
  return param;
}

double pget(const std::map<std::string, std::string>& m, const std::string& key, double def, double unit = 1) {
  auto it = m.find(key);
  if (it == m.end()) return def * unit;
  return atof(it->second.c_str()) * unit;
}
std::string sget(const std::map<std::string, std::string>& m, const std::string& key, const std::string& def) {
  auto it = m.find(key);
  return it == m.end() ? def : it->second;
}

// electron::fermi (electron.h:119-124)
double fermi(double t, double mu, double e) {
  double ebyt = (e - mu) / t;
  if (ebyt < -46) return 1;
  else if (ebyt > 46) return 0;
  else return 1. / (exp(ebyt) + 1);
}

struct zc {
  double x, y;
};
inline zc zmul(zc a, zc b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
inline zc zadd(zc a, zc b) { return {a.x + b.x, a.y + b.y}; }
inline zc zscale(double s, zc a) { return {a.x * s, a.y * s}; }
inline zc zconj(zc a) { return {a.x, -a.y}; }
inline zc zcis(double x) {
  return {cos(x), sin(x)};
}

bool read_file(const std::string& path, size_t expect, void* dst, std::string& why) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    why = path + " does not exist";
    return false;
  }
  fseek(f, 0L, SEEK_END);
  size_t sz = (size_t)ftell(f);
  rewind(f);
  if (sz != expect) {
    fclose(f);
    why = path + " size does not match expected size (" + std::to_string(sz) + " vs " + std::to_string(expect) + ")";
    return false;
  }
  size_t got = expect ? fread(dst, 1, expect, f) : 0;
  fclose(f);
  if (got != expect) {
    why = path + " short read";
    return false;
  }
  return true;
}

}  // namespace

// Carrier counting and chemical potentials. The impurity-level carriers of partially ionised
// impurities (Scatt_Param.h:82-94) are zero for the impurities accepted here.
namespace {

int isgn(double v) { return (0. < v) - (v < 0.); }  // sgn (electron.cpp:3-5)

// electron::compute_nfree (electron.cpp:578-596): e is [nk][nb], valence bands [0, nv)
double compute_nfree(bool isHole, double T, double mu, const double* e, int nk, int nb, int nv) {
  const int b0 = isHole ? 0 : nv, b1 = isHole ? nv : nb;
  double r = 0.;
  for (int ik = 0; ik < nk; ik++)
    for (int i = b0; i < b1; i++) {
      const double f = fermi(T, mu, e[(size_t)ik * nb + i]);
      if (!isHole) r += f;
      else r += (f - 1.);
    }
  return r;
}

// electron::find_mu by bisection in [emin, emax] (electron.cpp:537-572)
double find_mu_bisect(double carrier_bvk, bool is_excess, double T, double emin, double emax, const double* e, int nk,
                      int nb, int nv) {
  const bool isHole = carrier_bvk < 0;
  double lo = emin, hi = emax, result = 0, cnew;
  for (int niter = 1; niter <= 200; niter++) {
    result = 0.5 * (lo + hi);
    if (is_excess)
      cnew = compute_nfree(true, T, result, e, nk, nb, nv) + 0. + compute_nfree(false, T, result, e, nk, nb, nv) + 0.;
    else
      cnew = compute_nfree(isHole, T, result, e, nk, nb, nv) + 0.;
    if (fabs(cnew - carrier_bvk) < 1e-12) return result;
    if (cnew > carrier_bvk) hi = result;
    else lo = result;
  }
  return result;
}

// singdenmat_k::compute_nfree_eq (DenMat.cpp:198-225) over bands [b0, b1) of e_dm [nk][nb]
double nfree_eq(bool isHole, double T, double mu, const double* e, int nk, int nb, int b0, int b1) {
  double r = 0.;
  for (int ik = 0; ik < nk; ik++)
    for (int i = b0; i < b1; i++) {
      const double f = fermi(T, mu, e[(size_t)ik * nb + i]);
      if (!isHole) r += f;
      else r += (f - 1.);
    }
  return r;
}

// singdenmat_k::find_mu: damped search from mu0 (DenMat.cpp:150-197)
double find_mu_eq(bool isHole, double carrier_bvk, double T, double mu0, const double* e, int nk, int nb, int b0,
                  int b1) {
  double result = mu0, damp = 0.7, dmu = 5e-6, eoo = 1., eo = 1.;
  for (int step = 0;;) {
    const double cnew = nfree_eq(isHole, T, result, e, nk, nb, b0, b1) + 0.;
    const double excess = cnew - carrier_bvk;
    if (!(fabs(excess) > 1e-14)) break;
    if (fabs(excess) > fabs(eo) || fabs(excess) > fabs(eoo)) dmu *= damp;
    result -= isgn(excess) * dmu;
    if (step > 0 && isgn(excess) == isgn(eo)) {
      const double ratio = cnew / carrier_bvk;
      if (ratio < 1e-9) result -= (double)(isgn(excess) * 10) * T;
      else if (ratio < 1e-4) result -= (double)(isgn(excess) * 3) * T;
      else if (ratio < 0.1) result -= isgn(excess) * 0.7 * T;
    }
    if (dmu < 1e-16) break;
    eoo = eo;
    eo = excess;
    step++;
    if (step > 1e4) break;
  }
  return result;
}

}  // namespace

struct dmdh_system {
  std::map<std::string, std::string> pm;
  dmdh_info info;
  std::vector<double> e_dm, f_dm;
  std::vector<double> f_eq;         // [nk][nb_dm] with alg_ddmdteq
  std::vector<double> smat;         // complex [nk][3][nb_dm^2]
  std::vector<uint64_t> k1, k2;
  std::vector<double> P1, P2;       // complex [nkpair][nb^4], folded
  std::vector<double> dm0;          // complex [nk][nb_dm^2]
  std::vector<double> H;            // complex [nk][nb_dm^2] or empty
  double carrier_gs[3] = {0, 0, 0};  // eip.carrier_bvk_gs, ne_bvk_gs, nh_bvk_gs (electron.h:155-157)
  std::vector<std::pair<std::vector<double>, std::vector<double>>> imp;  // impurity P x |n_i V| (linear mode)
  int nimp = 0;                      // number of impurity densities (eip.ni.size())
  int sparse = 0;                    // alg_sparseP: the handle contracts the stored elements only
  double nfree = 0;                  // clp.nfreetot = |ne| + |nh| of set_mu_and_n (electron.h:157)
  // e-e model (eeMode): the descriptor for dmd_ee_attach and the arrays it points into
  int ee = 0;                        // 1: Pee_update, 2: Pee_fixed_at_eq
  int ee_freq = 0;                   // freq_update_ee_model (> 0: update between output steps)
  int64_t freq_measure = 1;          // S files every freq_measure-th step (report, DensityMatrix_Dynamics.h:323)
  int64_t freq_compute_tau = 10;     // tau files every freq_compute_tau-th step (:211, 230)
  int restart = 0;                   // restart = 1: state and time read from restart/
  int compute_tau_only = 0;          // report the tau files at t0 and stop (main.cpp:79)
  int print_tot_band = 0;            // the S files' per-band columns (observable.h:376-378)
  std::vector<double> kvec, U, f_win;
  dmd_ee_desc eed;
};

extern "C" {

const char* dmdh_error(void) { return g_err.c_str(); }

int dmdh_fermi(double T, double mu, const double* e, double* f, size_t n) {
  if ((!e || !f) && n) return DMD_E_ARG;
  for (size_t i = 0; i < n; ++i) f[i] = fermi(T, mu, e[i]);
  return DMD_OK;
}

// Worker threads that run one loop body over contiguous slices of [0, n), phase after phase (the
// caller's thread takes slice 0 and waits for the others); they sleep between phases.
class SlicePool {
 public:
  explicit SlicePool(unsigned nt) : nt_(nt < 1 ? 1 : nt) {
    for (unsigned w = 1; w < nt_; ++w) th_.emplace_back([this, w] { loop(w); });
  }
  ~SlicePool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void run(size_t n, const std::function<void(size_t, size_t)>& body) {
    if (nt_ == 1) {
      body(0, n);
      return;
    }
    {
      std::lock_guard<std::mutex> g(m_);
      body_ = &body;
      n_ = n;
      left_ = nt_ - 1;
      ++gen_;
    }
    cv_.notify_all();
    slice(0, n, body);
    std::unique_lock<std::mutex> l(m_);
    done_.wait(l, [this] { return left_ == 0; });
  }

 private:
  void slice(unsigned w, size_t n, const std::function<void(size_t, size_t)>& body) const {
    const size_t per = (n + nt_ - 1) / nt_, i0 = std::min(n, (size_t)w * per), i1 = std::min(n, i0 + per);
    if (i0 < i1) body(i0, i1);
  }
  void loop(unsigned w) {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(size_t, size_t)>* body;
      size_t n;
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        body = body_;
        n = n_;
      }
      slice(w, n, *body);
      {
        std::lock_guard<std::mutex> g(m_);
        if (--left_ == 0) done_.notify_one();
      }
    }
  }
  unsigned nt_;
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  const std::function<void(size_t, size_t)>* body_ = nullptr;
  size_t n_ = 0;
  unsigned left_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Fixed-step RK4 on the host around the GSL-callback entry, as a GSL-driven host runs it: every
// stage is one dmd_func call (its input copied to the device, dydt copied back) and the stage
// combinations are host loops: y_s = y + c h k, then y += h/6 (k1 + 2 k2 + 2 k3 + k4), split over
// up to 8 host threads (elementwise, so the result does not depend on the split).
int dmdh_rk4_func(dmd_handle* h, double t, double dt, int64_t nsteps, double* y, size_t n, double* work) {
  if (!h || !y || !work || n == 0 || nsteps < 0) return DMD_E_ARG;
  double* ys = work;
  double* k1 = work + n;
  double* k2 = work + 2 * n;
  double* k3 = work + 3 * n;
  double* k4 = work + 4 * n;
  const unsigned hw = std::thread::hardware_concurrency();
  SlicePool pool(n < (1u << 16) ? 1u : std::max(1u, std::min(8u, hw)));
  int rc = DMD_OK;
  for (int64_t s = 0; s < nsteps; ++s) {
    const double ts = t + (double)s * dt, hh = 0.5 * dt;
    auto stage = [&](const double* k, double c) {
      pool.run(n, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; ++i) ys[i] = y[i] + c * k[i];
      });
    };
    if ((rc = dmd_func(h, ts, y, k1))) return rc;
    stage(k1, hh);
    if ((rc = dmd_func(h, ts + hh, ys, k2))) return rc;
    stage(k2, hh);
    if ((rc = dmd_func(h, ts + hh, ys, k3))) return rc;
    stage(k3, dt);
    if ((rc = dmd_func(h, ts + dt, ys, k4))) return rc;
    const double c = dt / 6.0;
    pool.run(n, [&](size_t i0, size_t i1) {
      for (size_t i = i0; i < i1; ++i) y[i] += c * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]);
    });
  }
  return DMD_OK;
}

int dmdh_dm_bpert(int32_t nk, int32_t nb, const double* smat, const double* e, const double* f, double T,
                  const double Bpert[3], double t0, int32_t picture, double* dm) {
  if (nk <= 0 || nb <= 0 || !smat || !e || !f || !Bpert || !dm) return DMD_E_ARG;
  const double degthr = 1e-8;
  std::vector<zc> tmp((size_t)nb * nb);
  for (int ik = 0; ik < nk; ik++) {
    const zc* sk = (const zc*)smat + (size_t)ik * 3 * nb * nb;
    const double *ek = e + (size_t)ik * nb, *fk = f + (size_t)ik * nb;
    for (auto& v : tmp) v = {0, 0};
    for (int i = 0; i < nb; i++)
      for (int j = i; j < nb; j++) {
        zc H1 = zadd(zadd(zscale(Bpert[0], sk[i * nb + j]), zscale(Bpert[1], sk[nb * nb + i * nb + j])),
                     zscale(Bpert[2], sk[2 * nb * nb + i * nb + j]));
        double dfde;
        if (fabs(ek[i] - ek[j]) < degthr) {
          double favg = 0.5 * (fk[i] + fk[j]);
          dfde = favg * (favg - 1.) / T;
        } else {
          dfde = (fk[i] - fk[j]) / (ek[i] - ek[j]);
        }
        tmp[i * nb + j] = zscale(dfde, H1);
        if (i != j && picture == DMD_PICTURE_INTERACTION) tmp[i * nb + j] = zmul(tmp[i * nb + j], zcis((ek[i] - ek[j]) * t0));
        if (i < j) tmp[j * nb + i] = zconj(tmp[i * nb + j]);
      }
    for (int i = 0; i < nb; i++) tmp[i * nb + i] = zadd(tmp[i * nb + i], zc{fk[i], 0});
    // init_dm: Hermitian part (DenMat.cpp:74-78)
    zc* o = (zc*)dm + (size_t)ik * nb * nb;
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) o[i * nb + j] = zscale(0.5, zadd(tmp[i * nb + j], zconj(tmp[j * nb + i])));
  }
  return DMD_OK;
}

int dmdh_H_BS(int32_t nk, int32_t nb, const double* smat, const double B[3], const double* e, int32_t picture,
              double* H) {
  if (nk <= 0 || nb <= 0 || !smat || !B || !H) return DMD_E_ARG;
  for (int ik = 0; ik < nk; ik++) {
    const zc* sk = (const zc*)smat + (size_t)ik * 3 * nb * nb;
    zc* h = (zc*)H + (size_t)ik * nb * nb;
    for (int ij = 0; ij < nb * nb; ij++)
      h[ij] = zadd(zadd(zscale(B[0], sk[ij]), zscale(B[1], sk[nb * nb + ij])), zscale(B[2], sk[2 * nb * nb + ij]));
    if (picture == DMD_PICTURE_SCHRODINGER)
      for (int i = 0; i < nb; i++) h[i * nb + i].x += e[(size_t)ik * nb + i];
  }
  return DMD_OK;
}

// Linear operators from one source of P (electronphonon::add_Lscii_from_P1_P2 and
// add_Lscij_from_P1_P2 with fac2 = false, ElectronPhonon_linear.cpp:147-225), every pair in order.
// f is the window f_eq [nk][nb].
void lsc_add(int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P1, const zc* P2, const double* f,
             zc* Lscii, zc* Lij, zc* Lji, bool fac2 = false) {
  const int nb2 = nb * nb, nb4 = nb2 * nb2;
  auto sub = [](zc a, zc b) { return zc{a.x - b.x, a.y - b.y}; };
  auto add = [](zc a, zc b) { return zc{a.x + b.x, a.y + b.y}; };
  auto scl = [](double r, zc a) { return zc{a.x * r, a.y * r}; };  // complex * double
  auto cj = [](zc a) { return zc{a.x, -a.y}; };
  for (int64_t p = 0; p < npair; p++) {
    const int ik = (int)k1[p], jk = (int)k2[p];
    const zc* P1p = P1 + (size_t)p * nb4;
    const zc* P2p = P2 + (size_t)p * nb4;
    zc* Li = Lscii + (size_t)ik * nb4;
    zc* Lj = Lscii + (size_t)jk * nb4;
    for (int i1 = 0; i1 < nb; i1++)
      for (int i2 = 0; i2 < nb; i2++) {
        const int n12 = (i1 * nb + i2) * nb2;
        for (int ib = 0; ib < nb; ib++) {
          const int nbv = (ib * nb + i2) * nb2, i12ab = n12 + i1 * nb + ib;
          for (int i3 = 0; i3 < nb; i3++) {
            const int ib233 = nbv + i3 * nb + i3;
            Li[i12ab] = sub(Li[i12ab], scl(f[(size_t)jk * nb + i3], P1p[ib233]));
            if (jk > ik) Lj[i12ab] = sub(Lj[i12ab], scl(f[(size_t)ik * nb + i3], cj(P2p[ib233])));
          }
        }
        for (int ia = 0; ia < nb; ia++) {
          const int i1a = i1 * nb + ia, i12ab = n12 + ia * nb + i2;
          for (int i3 = 0; i3 < nb; i3++) {
            const int i331a = (i3 * nb + i3) * nb2 + i1a;
            Li[i12ab] = sub(Li[i12ab], scl(1 - f[(size_t)jk * nb + i3], P2p[i331a]));
            if (jk > ik) Lj[i12ab] = sub(Lj[i12ab], scl(1 - f[(size_t)ik * nb + i3], cj(P1p[i331a])));
          }
        }
      }
    zc* a = Lij + (size_t)p * nb4;
    zc* b = Lji + (size_t)p * nb4;
    for (int i1 = 0; i1 < nb; i1++)
      for (int i2 = 0; i2 < nb; i2++) {
        const int i12 = i1 * nb + i2, n12 = i12 * nb2;
        for (int iab = 0; iab < nb2; iab++) {
          const int i12ab = n12 + iab, iab12 = iab * nb2 + i12;
          const zc ca = add(scl(1 - f[(size_t)ik * nb + i1], P1p[i12ab]), scl(f[(size_t)ik * nb + i2], P2p[iab12]));
          const zc cb = add(scl(1 - f[(size_t)jk * nb + i1], cj(P2p[i12ab])), scl(f[(size_t)jk * nb + i2], cj(P1p[iab12])));
          a[i12ab] = add(a[i12ab], fac2 ? scl(2, ca) : ca);  // the exchange term doubles it (ElectronPhonon_linear.cpp:84)
          b[i12ab] = add(b[i12ab], fac2 ? scl(2, cb) : cb);
        }
      }
  }
}

// The e-e terms of the linear operators beyond P_ee: add_Lscij_from_P3_P4 and add_Lscij_from_P5_P6
// (ElectronPhonon_linear.cpp:199-245), every pair in order.
void lsc_add_p36(int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P3, const zc* P4,
                 const zc* P5, const zc* P6, const double* f, zc* Lij, zc* Lji) {
  const int nb2 = nb * nb, nb4 = nb2 * nb2;
  auto sub = [](zc a, zc b) { return zc{a.x - b.x, a.y - b.y}; };
  auto add = [](zc a, zc b) { return zc{a.x + b.x, a.y + b.y}; };
  auto scl = [](double r, zc a) { return zc{a.x * r, a.y * r}; };
  auto cj = [](zc a) { return zc{a.x, -a.y}; };
  for (int64_t p = 0; p < npair; p++) {
    const int ik = (int)k1[p], jk = (int)k2[p];
    const double *fi = f + (size_t)ik * nb, *fj = f + (size_t)jk * nb;
    zc* a = Lij + (size_t)p * nb4;
    zc* b = Lji + (size_t)p * nb4;
    if (P3) {
      const zc *a3 = P3 + (size_t)p * nb4, *a4 = P4 + (size_t)p * nb4;
      for (int i1 = 0; i1 < nb; i1++)
        for (int i2 = 0; i2 < nb; i2++) {
          const int i12 = i1 * nb + i2, n12 = i12 * nb2;
          for (int iab = 0; iab < nb2; iab++) {
            const int i12ab = n12 + iab, iab12 = iab * nb2 + i12;
            a[i12ab] = sub(a[i12ab], add(scl(1 - fi[i1], a3[i12ab]), scl(fi[i2], a4[i12ab])));
            b[i12ab] = sub(b[i12ab], add(scl(1 - fj[i1], cj(a4[iab12])), scl(fj[i2], cj(a3[iab12]))));
          }
        }
    }
    const zc *a5 = P5 + (size_t)p * nb4, *a6 = P6 + (size_t)p * nb4;
    for (int i1 = 0; i1 < nb; i1++)
      for (int i2 = 0; i2 < nb; i2++) {
        const int n12 = (i1 * nb + i2) * nb2, i21 = i2 * nb + i1;
        for (int ia = 0; ia < nb; ia++)
          for (int ib = 0; ib < nb; ib++) {
            const int i12ab = n12 + ia * nb + ib, iba21 = (ib * nb + ia) * nb2 + i21;
            a[i12ab] = sub(a[i12ab], add(scl(1 - fi[i1], a5[i12ab]), scl(fi[i2], a6[i12ab])));
            b[i12ab] = sub(b[i12ab], add(scl(1 - fj[i1], a5[iba21]), scl(fj[i2], a6[iba21])));
          }
      }
  }
}

// The e-e source of the linear operators, computed on the GPU: a temporary FP64 handle on the e-ph
// operators with the e-e model attached (the set-up screening and static RPA table), then P_ee and
// P3..P6 at the f_eq window (dmd_ee_linear_terms) with the screening density that
// coulomb_model::init(f_eq) gives when the model updates it (Coulomb_Model.h:532-544), the set-up one
// otherwise. T6: six complex [nkpair][nb^4] sets (P1ee, P2ee, P3, P4, P5, P6), scale_ee not applied.
static int ee_linear_terms(dmdh_system* s, const std::vector<double>& fw, std::vector<double>& T6) {
  dmd_desc d;
  dmdh_desc(s, DMD_PREC_F64, 0, &d);
  d.flags = DMD_FLAG_EE;
  d.Hcoh = nullptr;
  const dmdh_info& in = s->info;
  const int nb = in.bend - in.bstart;
  double nfree = s->eed.nfree;
  if (s->eed.update_screening) {
    double n = 0;
    for (int ik = 0; ik < in.nk; ik++)
      for (int b = 0; b < nb; b++) n += b < s->eed.nv ? (1 - fw[(size_t)ik * nb + b]) : fw[(size_t)ik * nb + b];
    nfree = n / (s->eed.nk_full * s->eed.cell_size);
  }
  dmd_handle* h = nullptr;
  int rc = dmd_create(&d, &h);
  if (rc) return err(rc, "the e-e source of the linear operators needs a GPU handle: dmd_create failed");
  const size_t n = (size_t)in.nkpair * nb * nb * nb * nb * 2;  // doubles per set
  if (!(rc = dmd_ee_attach(h, &s->eed)))
    rc = dmd_ee_linear_terms(h, fw.data(), nfree, T6.data(), T6.data() + n, T6.data() + 2 * n, T6.data() + 3 * n,
                             T6.data() + 4 * n, T6.data() + 5 * n);
  if (rc) {
    const std::string m = dmd_last_error(h);
    dmd_destroy(h);
    return err(rc, "the e-e source of the linear operators: " + m);
  }
  dmd_destroy(h);
  return DMD_OK;
}

int dmdh_load(const char* dir_c, dmdh_system** out) {
  if (!dir_c || !out) return err(DMD_E_ARG, "null argument");
  *out = nullptr;
  std::string dir(dir_c);
  std::unique_ptr<dmdh_system> s(new dmdh_system());
  dmdh_info& in = s->info;
  memset(&in, 0, sizeof(in));
  {
    std::ifstream fin(dir + "/param.in");
    if (!fin) return err(DMD_E_FILE, "input file param.in does not exist");
    s->pm = map_input(fin);
  }
  auto& pm = s->pm;
  // features outside this path are rejected explicitly
  const char* unsupported[] = {"alg_linearize_dPee", "alg_phenom_relax", "alg_semiclassical",
                               "alg_Pin_is_sparse", "alg_only_eimp", "alg_only_ee", "needL",
                               "alg_read_Bso", "gfac_normal_dist", "partial_ionized"};
  for (const char* k : unsupported)
    if (pget(pm, k, 0) != 0) return err(DMD_E_ARG, std::string(k) + " is not supported by the GB300 path");
  const bool linear = pget(pm, "alg_linearize", 0) != 0;
  s->sparse = pget(pm, "alg_sparseP", 0) != 0;  // the sparse contraction (DMD_FLAG_SPARSE, FP64)
  if (s->sparse && linear)  // parameters.cpp:434-435
    return err(DMD_E_ARG, "linearization does not support sparse matrices");
  if (s->sparse && sget(pm, "eeMode", "none") != "none")
    return err(DMD_E_ARG, "alg_sparseP with the e-e model is not supported by the GB300 path");
  if (linear && pget(pm, "alg_ddmdteq", 0) != 0)  // parameters.cpp:428-429
    return err(DMD_E_ARG, "if master equation is linearized, ddmdt_eq is not needed");
  if (sget(pm, "code", "jdftx") != "jdftx" || sget(pm, "material_model", "none") != "none")
    return err(DMD_E_ARG, "only code = jdftx, material_model = none");
  if (pget(pm, "laserA", pget(pm, "pumpA0", 0)) > 0) return err(DMD_E_ARG, "laser is not supported");
  const std::string ee_mode = sget(pm, "eeMode", "none"), scr_mode = sget(pm, "scrMode", "none");
  if (ee_mode == "none" && scr_mode != "none") return err(DMD_E_ARG, "screening without the e-e model is not supported");
  if (ee_mode != "none") {  // the e-e model (parameters.cpp:479-500, Scatt_Param.h:21-47)
    if (ee_mode != "Pee_update" && ee_mode != "Pee_fixed_at_eq")
      return err(DMD_E_ARG, "eeMode must be none, Pee_fixed_at_eq or Pee_update");
    if (scr_mode != "medium") return err(DMD_E_ARG, "the e-e model needs scrMode = medium");
    const std::string f = sget(pm, "scrFormula", "RPA");
    if (f == "lindhard")  // the reference builds no vq table for it (init_RPA runs for RPA only)
      return err(DMD_E_ARG, "scrFormula lindhard has no static vq table in the reference (Coulomb_Model.h:537-545)");
    if (f != "unscreened" && f != "debye" && f != "Bechstedt" && f != "RPA")
      return err(DMD_E_ARG, "scrFormula " + f + " is not supported (unscreened, debye, Bechstedt, RPA are)");
    // dynamic screening (Scatt_Param.h:20-49): static, or the plasmon-pole approximation with RPA
    const std::string dyn = sget(pm, "dynamic_screening", "static");
    if (dyn != "static" && dyn != "ppa")
      return err(DMD_E_ARG, "dynamic_screening " + dyn + " is not supported (static, ppa are)");
    if (dyn == "static" && pget(pm, "dynamic_screening_ee_two_freqs", 0) != 0)
      return err(DMD_E_ARG, "only for dynamic screening, dynamic_screening_ee_two_freqs can be true");
    if (dyn != "static" && f != "RPA") return err(DMD_E_ARG, "debye and Bechstedt models are in static limit");
    if (dyn != "static" && pget(pm, "alg_linearize", 0) != 0)
      return err(DMD_E_ARG, "the linearized e-e source is supported with static screening only");
    const std::string ppam = sget(pm, "ppamodel", "gn");
    if (ppam != "gn" && ppam != "hl") return err(DMD_E_ARG, "ppamodel is invalid");
    if (pget(pm, "eppa_screening", 0) < 0) return err(DMD_E_ARG, "eppa must >= 0");
    if (pget(pm, "smearing_screening", 0) < 0) return err(DMD_E_ARG, "smearing must >= 0");
    if (pget(pm, "alg_summode", 1) == 0) return err(DMD_E_ARG, "the e-e model needs alg_summode");
    const double fe = pget(pm, "freq_update_ee_model", 0), fi = pget(pm, "freq_update_eimp_model", 0);
    if (ee_mode == "Pee_update" && fe == 0)  // parameters.cpp:483-484
      return err(DMD_E_ARG, "want to update Pee but set freq_update_ee_model as 0");
    if (fi != fe)  // parameters.cpp:499-500
      return err(DMD_E_ARG, "freq_update_eimp_model is the same as freq_update_ee_model in current version");
    s->ee = ee_mode == "Pee_update" ? 1 : 2;
    s->ee_freq = ee_mode == "Pee_update" && fe > 0 ? (int)fe : 0;
  }
  if (sget(pm, "alg_scatt", "lindblad") != "lindblad") return err(DMD_E_ARG, "alg_scatt must be lindblad");
  if (pget(pm, "alg_eph_sepr_eh", 1) != 0 && pget(pm, "alg_eph_need_elec", 1) == 0)
    return err(DMD_E_ARG, "hole-only e-ph data is not supported");
  // ldbd_size.dat (electron.cpp:100-133, ElectronPhonon.cpp:132-177, parameters.cpp:7-23)
  FILE* fp = fopen((dir + "/ldbd_data/ldbd_size.dat").c_str(), "r");
  if (!fp) return err(DMD_E_FILE, "ldbd_data/ldbd_size.dat does not exist");
  char line[512];
  std::vector<std::string> lines;
  while (fgets(line, sizeof line, fp)) lines.push_back(line);
  fclose(fp);
  if (lines.size() < 8) return err(DMD_E_FILE, "ldbd_size.dat is too short");
  int nb, nv, bStart_dm, bEnd_dm, bStart_eph, bEnd_eph, i7, i8, i9;
  if (sscanf(lines[1].c_str(), "%d %d %d %d %d %d %d %d %d", &nb, &nv, &bStart_dm, &bEnd_dm, &bStart_eph, &bEnd_eph, &i7,
             &i8, &i9) < 6)
    return err(DMD_E_FILE, "ldbd_size.dat line 2");
  double nk_full;
  int nk, km0, km1, km2;
  if (sscanf(lines[2].c_str(), "%le %d %d %d %d", &nk_full, &nk, &km0, &km1, &km2) < 2)
    return err(DMD_E_FILE, "ldbd_size.dat line 3");
  int nkpair;
  if (sscanf(lines[3].c_str(), "%d", &nkpair) != 1) return err(DMD_E_FILE, "ldbd_size.dat line 4");
  double T, mu_min, mu_max, mu_file;
  if (sscanf(lines[5].c_str(), "%le", &T) != 1) return err(DMD_E_FILE, "ldbd_size.dat line 6");
  if (sscanf(lines[6].c_str(), "%lg %lg %lg", &mu_min, &mu_max, &mu_file) != 3) return err(DMD_E_FILE, "line 7");
  if (nv < 0 || nv > nb || bStart_dm < 0 || bStart_dm > bEnd_dm || bEnd_dm > nb || bStart_eph < bStart_dm ||
      bStart_eph > bEnd_eph || bEnd_eph > bEnd_dm || nk <= 0 || nkpair < 0)
    return err(DMD_E_FILE, "inconsistent band ranges in ldbd_size.dat");
  const int nb_dm = bEnd_dm - bStart_dm;
  const int bs = bStart_eph - bStart_dm, be = bEnd_eph - bStart_dm, nbw = be - bs;
  if (nb_dm > 8 || nbw < 1 || nbw > 4) return err(DMD_E_ARG, "band counts out of the supported range");
  in.nk = nk;
  in.nb_dm = nb_dm;
  in.bstart = bs;
  in.bend = be;
  in.nb_total = nb;
  in.nv_dm = std::max(nv - bStart_dm, 0);  // electron.cpp:114
  in.nkpair = nkpair;
  in.nk_full = nk_full;
  in.temperature = T;
  in.mu = pget(pm, "mu", mu_file / kEV, kEV);
  in.prefac_eph = 2 * M_PI / nk_full;
  // lattice (lattice.h:15-56)
  int dim = 3;
  double R[3][3] = {{0}};
  if (FILE* fr = fopen((dir + "/ldbd_data/ldbd_R.dat").c_str(), "r")) {
    if (fscanf(fr, "%d", &dim) != 1) dim = 3;
    for (int i = 0; i < 3; i++)
      if (fscanf(fr, "%lf %lf %lf", &R[i][0], &R[i][1], &R[i][2]) != 3) { fclose(fr); return err(DMD_E_FILE, "ldbd_R.dat"); }
    fclose(fr);
  } else {
    return err(DMD_E_FILE, "ldbd_data/ldbd_R.dat does not exist");
  }
  dim = (int)pget(pm, "dim", dim);
  // det(R) = box(row0, row1, row2) = dot(row0, cross(row1, row2)) (comm/matrix3.h:276, vector3.h:117-126)
  const double cx = R[1][1] * R[2][2] - R[1][2] * R[2][1], cy = R[1][2] * R[2][0] - R[1][0] * R[2][2],
               cz = R[1][0] * R[2][1] - R[1][1] * R[2][0];
  const double volume = fabs(R[0][0] * cx + R[0][1] * cy + R[0][2] * cz);
  double cell = volume;
  if (dim == 2) cell = volume / R[2][2];
  if (dim == 1) cell = R[2][2];
  if (dim == 0) cell = 1;
  if (dim == 2 && pget(pm, "thickness", 0) > 1e-6) {
    // thickness only affects 2D volume-normalised analysis, not the cell size of observables
  }
  in.cell_size = cell;
  in.cell_size_cmd = cell * std::pow(kBohr2cm, dim);
  in.ob_prefac = (1. / nk_full) / in.cell_size_cmd;
  // energies and occupations (electron.cpp:171-207)
  std::string why;
  std::vector<double> e((size_t)nk * nb);
  if (!read_file(dir + "/ldbd_data/ldbd_ek.bin", e.size() * 8, e.data(), why)) return err(DMD_E_FILE, why);
  const double scissor = pget(pm, "scissor", 0, kEV);
  if (scissor != 0)
    for (int ik = 0; ik < nk; ik++)
      for (int i = nv; i < nb; i++) e[(size_t)ik * nb + i] = 1 * e[(size_t)ik * nb + i] + scissor;
  s->e_dm.resize((size_t)nk * nb_dm);
  s->f_dm.resize((size_t)nk * nb_dm);
  for (int ik = 0; ik < nk; ik++)
    for (int b = 0; b < nb_dm; b++) s->e_dm[(size_t)ik * nb_dm + b] = e[(size_t)ik * nb + bStart_dm + b];
  // electron constructor energy range (electron.h:94-105) and set_mu_and_n (electron.h:141-160)
  {
    const int nvd = in.nv_dm;
    double emax = -DBL_MAX, ecmin = DBL_MAX, evmax = -DBL_MAX, emin = DBL_MAX;
    for (int ik = 0; ik < nk; ik++) {
      for (int b = nvd; b < nb_dm; b++) {
        const double v = s->e_dm[(size_t)ik * nb_dm + b];
        if (v > emax) emax = v;
        if (v < ecmin) ecmin = v;
      }
      for (int b = 0; b < nvd; b++) {
        const double v = s->e_dm[(size_t)ik * nb_dm + b];
        if (v > evmax) evmax = v;
        if (v < emin) emin = v;
      }
    }
    if (nb_dm == nvd) emax = evmax + 1;
    if (nvd == 0) emin = ecmin - 1;
    const double cd = pget(pm, "carrier_density", 0, std::pow(kBohr2cm, dim));
    const bool excess = pget(pm, "carrier_density_means_excess_density", 0) != 0;
    if (cd != 0 && !excess) in.mu = find_mu_bisect(cd * nk_full * cell, false, T, emin, emax, e.data(), nk, nb, nv);
    if (excess) in.mu = find_mu_bisect(cd * nk_full * cell, true, T, emin, emax, e.data(), nk, nb, nv);
    const double ne = compute_nfree(false, T, in.mu, e.data(), nk, nb, nv) / nk_full / cell;
    const double nh = compute_nfree(true, T, in.mu, e.data(), nk, nb, nv) / nk_full / cell;
    const double nei = 0. / nk_full / cell, nhi = 0. / nk_full / cell;
    s->nfree = fabs(ne) + fabs(nh);
    double gs = fabs(ne + nei) > fabs(nh + nhi) ? ne + nei : nh + nhi;
    s->carrier_gs[0] = gs * nk_full * cell;
    s->carrier_gs[1] = ne * nk_full * cell;
    s->carrier_gs[2] = nh * nk_full * cell;
  }
  for (int ik = 0; ik < nk; ik++)
    for (int b = 0; b < nb_dm; b++)
      s->f_dm[(size_t)ik * nb_dm + b] = fermi(T, in.mu, e[(size_t)ik * nb + bStart_dm + b]);
  // spin matrices (electron.cpp:284-314)
  s->smat.resize((size_t)nk * 3 * nb_dm * nb_dm * 2);
  if (!read_file(dir + "/ldbd_data/ldbd_smat.bin", s->smat.size() * 8, s->smat.data(), why)) return err(DMD_E_FILE, why);
  if (pget(pm, "alg_set_scv_zero", 0) != 0) {
    const int nvd = std::max(nv - bStart_dm, 0);
    zc* sm = (zc*)s->smat.data();
    for (size_t k = 0; k < (size_t)nk * 3; k++)
      for (int i = 0; i < nvd; i++)
        for (int j = nvd; j < nb_dm; j++) {
          sm[k * nb_dm * nb_dm + i * nb_dm + j] = {0, 0};
          sm[k * nb_dm * nb_dm + j * nb_dm + i] = {0, 0};
        }
  }
  // k-pairs and P (ElectronPhonon.cpp:182-253)
  s->k1.resize(nkpair);
  s->k2.resize(nkpair);
  if (!read_file(dir + "/ldbd_data/ldbd_kpair_k1st.bin", (size_t)nkpair * 8, s->k1.data(), why) ||
      !read_file(dir + "/ldbd_data/ldbd_kpair_k2nd.bin", (size_t)nkpair * 8, s->k2.data(), why))
    return err(DMD_E_FILE, why);
  for (int p = 0; p < nkpair; p++)
    if (s->k1[p] >= (uint64_t)nk || s->k2[p] >= (uint64_t)nk) return err(DMD_E_FILE, "k-pair index out of range");
  const size_t np4 = (size_t)nkpair * nbw * nbw * nbw * nbw;
  s->P1.assign(2 * np4, 0.0);
  s->P2.assign(2 * np4, 0.0);
  const double scale_scatt = pget(pm, "scale_scatt", 1.);
  if (pget(pm, "alg_eph_enable", 1) != 0) {
    if (!read_file(dir + "/ldbd_data/ldbd_P1_lindblad.bin", np4 * 16, s->P1.data(), why) ||
        !read_file(dir + "/ldbd_data/ldbd_P2_lindblad.bin", np4 * 16, s->P2.data(), why))
      return err(DMD_E_FILE, why);
    const double scale_eph = pget(pm, "scale_eph", scale_scatt);
    if (scale_eph != 1.)
      for (size_t i = 0; i < 2 * np4; i++) {
        s->P1[i] = s->P1[i] * scale_eph;
        s->P2[i] = s->P2[i] * scale_eph;
      }
  }
  // ab-initio e-imp operators, one per impurity_density{,2,3,...} (parameters.cpp:213-228)
  const double scale_ei = pget(pm, "scale_ei", scale_scatt);
  std::vector<double> A1, A2;
  in.eimp_fraction = 0;
  for (int iD = 0;; iD++) {
    const std::string nm = iD == 0 ? "" : std::to_string(iD + 1);
    const double ni = pget(pm, "impurity_density" + nm, 0, std::pow(kBohr2cm, dim));
    if (ni == 0) break;
    if (sget(pm, "impMode" + nm, "model_ionized") != "ab_neutral")
      return err(DMD_E_ARG, "only impMode = ab_neutral is supported");
    if (s->sparse)  // parameters.cpp:472-473
      return err(DMD_E_ARG, "ab initio neutral e-imp does not support sparse matrices");
    s->nimp = iD + 1;
    const double fraction = fabs(ni * cell);  // electronimpurity ctor (ElectronImpurity.h:18)
    if (iD == 0) in.eimp_fraction = fraction;
    A1.assign(2 * np4, 0.0);
    A2.assign(2 * np4, 0.0);
    const std::string sfx = "_D" + std::to_string(iD + 1);
    if (!read_file(dir + "/ldbd_data/ldbd_P1_lindblad" + sfx + ".bin", np4 * 16, A1.data(), why) ||
        !read_file(dir + "/ldbd_data/ldbd_P2_lindblad" + sfx + ".bin", np4 * 16, A2.data(), why))
      return err(DMD_E_FILE, why);
    for (size_t i = 0; i < 2 * np4; i++) {
      double a1 = A1[i] * fraction, a2 = A2[i] * fraction;
      if (scale_ei != 1.) {
        a1 = a1 * scale_ei;
        a2 = a2 * scale_ei;
      }
      if (linear) {  // kept apart: each source adds its own linear operators (ElectronPhonon_linear.cpp:57-79)
        A1[i] = a1;
        A2[i] = a2;
      } else {
        s->P1[i] = s->P1[i] + a1;
        s->P2[i] = s->P2[i] + a2;
      }
    }
    if (linear) s->imp.push_back({A1, A2});
  }
  // time and picture parameters (parameters.cpp:99-106, 283-336, 359-367)
  const std::string pic = sget(pm, "alg_picture", "interaction");
  in.picture = (pic == "schrodinger" || pic == "non-interaction") ? DMD_PICTURE_SCHRODINGER : DMD_PICTURE_INTERACTION;
  in.expt = (int)pget(pm, "alg_expt", 1);
  if (in.picture == DMD_PICTURE_SCHRODINGER && in.expt) return err(DMD_E_ARG, "in schrodinger picture, alg_expt must be false");
  const bool restart = pget(pm, "restart", 0) != 0;
  s->restart = restart ? 1 : 0;
  s->compute_tau_only = pget(pm, "compute_tau_only", 0) != 0 ? 1 : 0;
  s->print_tot_band = pget(pm, "print_tot_band", 0) != 0 ? 1 : 0;
  in.t0 = pget(pm, "t0", 0., kFs);
  if (restart) {
    FILE* ft = fopen((dir + "/restart/time_restart.dat").c_str(), "r");
    if (!ft) return err(DMD_E_FILE, "restart needs restart/time_restart.dat");
    if (fscanf(ft, "%le", &in.t0) != 1) { fclose(ft); return err(DMD_E_FILE, "time_restart.dat"); }
    fclose(ft);
  }
  in.tend = pget(pm, "tend", 0., kFs);
  in.tstep = pget(pm, "tstep", 1., kFs);
  in.ode_hstart = pget(pm, "ode_hstart", 1e-3, kFs);
  in.ode_hmin = pget(pm, "ode_hmin", 0, kFs);
  in.ode_hmax = pget(pm, "ode_hmax", in.tstep / kFs, kFs);
  in.ode_epsabs = pget(pm, "ode_epsabs", 1e-8);
  // measurement frequencies (parameters.cpp:324-326); DMD takes them modulo, so they must be >= 1
  s->freq_measure = (int64_t)pget(pm, "freq_measure", 1);
  s->freq_compute_tau = (int64_t)pget(pm, "freq_compute_tau", (double)(int64_t)pget(pm, "freq_measure_ene", 10));
  if (s->freq_measure < 1 || s->freq_compute_tau < 1) return err(DMD_E_ARG, "freq_measure and freq_compute_tau must be >= 1");
  const std::string om = sget(pm, "alg_ode_method", "rkf45");
  in.ode_method = om == "rkf45" ? 0 : om == "euler" ? 1 : om == "rk4" ? 2 : -1;
  if (in.ode_method < 0) return err(DMD_E_ARG, "alg_ode_method must be rkf45, euler or rk4");
  in.Bpert[0] = pget(pm, "Bxpert", 0., kTesla2au);
  in.Bpert[1] = pget(pm, "Bypert", 0., kTesla2au);
  in.Bpert[2] = pget(pm, "Bzpert", 0., kTesla2au);
  in.B[0] = pget(pm, "Bx", 0., kTesla2au);
  in.B[1] = pget(pm, "By", 0., kTesla2au);
  in.B[2] = pget(pm, "Bz", 0., kTesla2au);
  // initial density matrix (electron.cpp:62-98, DenMat.cpp:65-81, 301-317)
  s->dm0.resize((size_t)nk * nb_dm * nb_dm * 2);
  if (restart) {
    if (!read_file(dir + "/restart/denmat_restart.bin", s->dm0.size() * 8, s->dm0.data(), why)) return err(DMD_E_FILE, why);
  } else {
    int rc = dmdh_dm_bpert(nk, nb_dm, s->smat.data(), s->e_dm.data(), s->f_dm.data(), T, in.Bpert, in.t0, in.picture,
                           s->dm0.data());
    if (rc) return err(rc, "dm_Bpert");
  }
  // equilibrium occupations for the drift subtraction (DensityMatrix_Dynamics.h:58-63 ->
  // singdenmat_k::set_dm_eq, DenMat.cpp:97-148, on the initial or restart state)
  in.mue = in.muh = in.mu;
  if (pget(pm, "alg_ddmdteq", 0) != 0 || linear) {
    in.ddmdteq = linear ? 0 : 1;
    in.linear = linear ? 1 : 0;
    const int nvd = in.nv_dm;
    const zc* dm = (const zc*)s->dm0.data();
    double mus[2] = {in.mu, in.mu};
    for (int pass = 0; pass < 2; pass++) {
      const bool isHole = pass == 1;
      if (!isHole && !(nb_dm > nvd)) continue;
      if (isHole && !(nvd > 0)) continue;
      const int b0 = isHole ? 0 : nvd, b1 = isHole ? nvd : nb_dm;
      double nfree = 0.;
      for (int ik = 0; ik < nk; ik++)
        for (int i = b0; i < b1; i++) {
          if (!isHole) nfree += dm[(size_t)ik * nb_dm * nb_dm + i * nb_dm + i].x;
          else nfree += (dm[(size_t)ik * nb_dm * nb_dm + i * nb_dm + i].x - 1.);
        }
      // elecimpParam::carrier_bvk_ex (Scatt_Param.h:63-68)
      const double* gs = s->carrier_gs;
      double target;
      if (s->nimp == 0 || (gs[0] > 0 && isHole) || (gs[0] < 0 && !isHole)) target = nfree;
      else if (gs[0] < 0 && isHole) target = gs[0] + (nfree - gs[2]);
      else if (gs[0] > 0 && !isHole) target = gs[0] + (nfree - gs[1]);
      else return err(DMD_E_ARG, "alg_ddmdteq with impurities needs a non-zero ground-state carrier density");
      double m = find_mu_eq(isHole, target, T, mus[pass], s->e_dm.data(), nk, nb_dm, b0, b1);
      if (pget(pm, "DEBUG", 0) != 0) m = mus[pass];
      mus[pass] = m;
    }
    in.mue = mus[0];
    in.muh = mus[1];
    s->f_eq.resize((size_t)nk * nb_dm);
    for (int ik = 0; ik < nk; ik++)
      for (int i = 0; i < nb_dm; i++)
        s->f_eq[(size_t)ik * nb_dm + i] = fermi(T, i < nvd ? in.muh : in.mue, s->e_dm[(size_t)ik * nb_dm + i]);
  }
  if (s->ee) {
    // elecelec_model / coulomb_model inputs (ElecElec_Model.h:22-37, Coulomb_Model.h:415-424): the
    // k-points and U (electron.cpp:134-146, 388-410; U's partial layout [nk][nb_wannier][nb_eph] is
    // the one the reference reads, see its size check), the reciprocal metric (lattice.h:41-42)
    int nbwan = 0;
    if (sscanf(lines[1].c_str(), "%*d %*d %*d %*d %*d %*d %d", &nbwan) != 1 || nbwan < nbw)
      return err(DMD_E_FILE, "ldbd_size.dat: nb_wannier");
    s->kvec.resize((size_t)nk * 3);
    s->U.resize((size_t)nk * nbwan * nbw * 2);
    if (!read_file(dir + "/ldbd_data/ldbd_kvec.bin", s->kvec.size() * 8, s->kvec.data(), why) ||
        !read_file(dir + "/ldbd_data/ldbd_Umat.bin", s->U.size() * 8, s->U.data(), why))
      return err(DMD_E_FILE, why);
    s->f_win.resize((size_t)nk * nbw);
    for (int ik = 0; ik < nk; ik++)
      for (int b = 0; b < nbw; b++) s->f_win[(size_t)ik * nbw + b] = s->f_dm[(size_t)ik * nb_dm + bs + b];
    // GGT = Gvec Gvec^T, Gvec = 2 pi inv(R), inv = adjugate / det (comm/matrix3.h:248-284)
    double adj[3][3], G[3][3];
    const double c0[3] = {R[1][1] * R[2][2] - R[1][2] * R[2][1], R[1][2] * R[2][0] - R[1][0] * R[2][2],
                          R[1][0] * R[2][1] - R[1][1] * R[2][0]};
    const double c1[3] = {R[2][1] * R[0][2] - R[2][2] * R[0][1], R[2][2] * R[0][0] - R[2][0] * R[0][2],
                          R[2][0] * R[0][1] - R[2][1] * R[0][0]};
    const double c2[3] = {R[0][1] * R[1][2] - R[0][2] * R[1][1], R[0][2] * R[1][0] - R[0][0] * R[1][2],
                          R[0][0] * R[1][1] - R[0][1] * R[1][0]};
    const double det = R[0][0] * c0[0] + R[0][1] * c0[1] + R[0][2] * c0[2];
    for (int i = 0; i < 3; i++) {
      adj[i][0] = c0[i];
      adj[i][1] = c1[i];
      adj[i][2] = c2[i];
    }
    const double sdet = 1. / det;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) G[i][j] = (adj[i][j] * sdet) * (2. * M_PI);
    dmd_ee_desc& ee = s->eed;
    memset(&ee, 0, sizeof(ee));
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double acc = 0;
        for (int k = 0; k < 3; k++) acc += G[i][k] * G[j][k];
        ee.GGT[i * 3 + j] = acc;
      }
    double degauss = 0, ndegauss = 0;
    if (sscanf(lines[7].c_str(), "%lg %lg", &degauss, &ndegauss) != 2) return err(DMD_E_FILE, "ldbd_size.dat line 8");
    degauss = pget(pm, "degauss", degauss / kEV, kEV);  // parameters.cpp:131-140
    ndegauss = pget(pm, "ndegauss", ndegauss);
    const std::string f = sget(pm, "scrFormula", "RPA");
    ee.nbw = nbwan;
    ee.kvec = s->kvec.data();
    ee.kmesh[0] = km0;
    ee.kmesh[1] = km1;
    ee.kmesh[2] = km2;
    ee.U = s->U.data();
    ee.f = s->f_win.data();
    ee.cell_size = cell;
    ee.nk_full = nk_full;
    ee.temperature = T;
    ee.eps_background = pget(pm, "epsilon_background", 1);
    ee.meff = pget(pm, "meff_screening", 1);
    ee.formula = f == "unscreened" ? DMD_SCREEN_UNSCREENED
                 : f == "debye"    ? DMD_SCREEN_DEBYE
                 : f == "RPA"      ? DMD_SCREEN_RPA
                                   : DMD_SCREEN_BECHSTEDT;
    ee.nfree = s->nfree;
    ee.update_screening = pget(pm, "update_screening", 1) != 0;
    ee.nv = in.nv_dm - bs;  // coul_model->nv (Coulomb_Model.h:418)
    ee.degauss = pget(pm, "degauss_ee", degauss / kEV, kEV);
    ee.ethr = degauss * ndegauss;
    ee.antisymmetry = pget(pm, "ee_antisymmetry", 0) != 0;
    ee.scale = pget(pm, "scale_ee", scale_scatt);
    ee.every_rhs = s->ee == 1 && pget(pm, "freq_update_ee_model", 0) < 0;
    ee.dynamic = sget(pm, "dynamic_screening", "static") == "ppa";  // parameters.cpp:196-204
    ee.ppa_gn = sget(pm, "ppamodel", "gn") == "gn";
    ee.eppa = pget(pm, "eppa_screening", 0);
    ee.smearing = pget(pm, "smearing_screening", 0, kEV);
    ee.two_freqs = pget(pm, "dynamic_screening_ee_two_freqs", 0) != 0;
  }
  if (linear) {
    // electronphonon::set_Lsc (ElectronPhonon_linear.cpp:3-31): the e-ph operators, each impurity's,
    // then Lscii onto the diagonal pairs; the linear operators replace P1, P2
    std::vector<double> fw((size_t)nk * nbw);
    for (int ik = 0; ik < nk; ik++)
      for (int b = 0; b < nbw; b++) fw[(size_t)ik * nbw + b] = s->f_eq[(size_t)ik * nb_dm + bs + b];
    const size_t nb4 = (size_t)nbw * nbw * nbw * nbw;
    std::vector<double> Lii(2 * (size_t)nk * nb4, 0.0), Lij(2 * np4, 0.0), Lji(2 * np4, 0.0);
    lsc_add(nbw, nkpair, s->k1.data(), s->k2.data(), (const zc*)s->P1.data(), (const zc*)s->P2.data(), fw.data(),
            (zc*)Lii.data(), (zc*)Lij.data(), (zc*)Lji.data());
    for (auto& a : s->imp)
      lsc_add(nbw, nkpair, s->k1.data(), s->k2.data(), (const zc*)a.first.data(), (const zc*)a.second.data(), fw.data(),
              (zc*)Lii.data(), (zc*)Lij.data(), (zc*)Lji.data());
    if (s->ee) {  // add_Lsc_contrib("ee") (ElectronPhonon_linear.cpp:17-22, 44-100), computed on the GPU
      std::vector<double> T6((size_t)6 * np4 * 2, 0.0);
      int rc = ee_linear_terms(s.get(), fw, T6);
      if (rc) return rc;
      const double sc = s->eed.scale;
      if (sc != 1.)
        for (size_t i = 0; i < T6.size(); i += 2) {  // complex(scale_ee, 0) * P
          const double x = T6[i], y = T6[i + 1];
          T6[i] = sc * x - 0 * y;
          T6[i + 1] = sc * y + 0 * x;
        }
      const zc* T = (const zc*)T6.data();
      const size_t n4 = np4;  // complex elements per operator set
      const bool anti = s->eed.antisymmetry != 0, fixed = s->ee == 2;
      lsc_add(nbw, nkpair, s->k1.data(), s->k2.data(), T, T + n4, fw.data(), (zc*)Lii.data(), (zc*)Lij.data(),
              (zc*)Lji.data(), anti);
      if (!fixed)
        lsc_add_p36(nbw, nkpair, s->k1.data(), s->k2.data(), anti ? nullptr : T + 2 * n4, T + 3 * n4, T + 4 * n4,
                    T + 5 * n4, fw.data(), (zc*)Lij.data(), (zc*)Lji.data());
    }
    for (int p = 0; p < nkpair; p++) {
      if (s->k1[p] != s->k2[p]) continue;
      const zc* x = (const zc*)Lii.data() + s->k1[p] * nb4;
      zc* a = (zc*)Lij.data() + (size_t)p * nb4;
      zc* b = (zc*)Lji.data() + (size_t)p * nb4;
      for (size_t e = 0; e < nb4; e++) {  // axbyc(L, Lscii, n, c1, c1): L += Lscii + 0
        const zc t = {x[e].x + 0.0, x[e].y + 0.0};
        a[e] = {a[e].x + t.x, a[e].y + t.y};
        b[e] = {b[e].x + t.x, b[e].y + t.y};
      }
    }
    s->P1.swap(Lij);
    s->P2.swap(Lji);
    s->imp.clear();
  }
  // coherent Hamiltonian (main.cpp:51)
  const double Blen = sqrt(in.B[0] * in.B[0] + in.B[1] * in.B[1] + in.B[2] * in.B[2]);
  if (Blen > 1e-10) {
    s->H.resize((size_t)nk * nb_dm * nb_dm * 2);
    dmdh_H_BS(nk, nb_dm, s->smat.data(), in.B, s->e_dm.data(), in.picture, s->H.data());
    in.has_H = 1;
  }
  *out = s.release();
  return DMD_OK;
}

void dmdh_free(dmdh_system* s) { delete s; }

int dmdh_info_get(const dmdh_system* s, dmdh_info* info) {
  if (!s || !info) return DMD_E_ARG;
  *info = s->info;
  return DMD_OK;
}

int dmdh_desc(const dmdh_system* s, int32_t precision, int32_t device, dmd_desc* d) {
  if (!s || !d) return DMD_E_ARG;
  memset(d, 0, sizeof(*d));
  d->nk = s->info.nk;
  d->nb_dm = s->info.nb_dm;
  d->bstart = s->info.bstart;
  d->bend = s->info.bend;
  d->nkpair = s->info.nkpair;
  d->prefac_eph = s->info.prefac_eph;
  d->e_dm = s->e_dm.data();
  d->k1st = s->k1.data();
  d->k2nd = s->k2.data();
  d->P1 = s->P1.data();
  d->P2 = s->P2.data();
  d->Hcoh = s->H.empty() ? nullptr : s->H.data();
  d->picture = s->info.picture;
  d->expt = s->info.expt;
  d->precision = precision;
  d->device = device;
  // (linearized: the e-e term is part of the linear operators, no model on the handle)
  d->flags = (s->info.linear ? DMD_FLAG_LINEAR : 0u) | (s->ee && !s->info.linear ? DMD_FLAG_EE : 0u) |
             (s->sparse ? DMD_FLAG_SPARSE : 0u);
  d->f_ref = s->f_eq.empty() ? s->f_dm.data() : s->f_eq.data();
  return DMD_OK;
}

int dmdh_get_dm0(const dmdh_system* s, double* dm0) {
  if (!s || !dm0) return DMD_E_ARG;
  memcpy(dm0, s->dm0.data(), s->dm0.size() * 8);
  return DMD_OK;
}
int dmdh_get_f(const dmdh_system* s, double* f) {
  if (!s || !f) return DMD_E_ARG;
  memcpy(f, s->f_dm.data(), s->f_dm.size() * 8);
  return DMD_OK;
}
int dmdh_get_f_eq(const dmdh_system* s, double* f_eq) {
  if (!s || !f_eq) return DMD_E_ARG;
  if (s->f_eq.empty()) return err(DMD_E_ARG, "alg_ddmdteq and alg_linearize are off: no equilibrium occupations");
  memcpy(f_eq, s->f_eq.data(), s->f_eq.size() * 8);
  return DMD_OK;
}

int dmdh_ee_desc(const dmdh_system* s, dmd_ee_desc* ee, int32_t* on) {
  if (!s || !ee || !on) return DMD_E_ARG;
  *on = s->ee ? 1 : 0;
  if (s->ee) *ee = s->eed;
  return DMD_OK;
}

int dmdh_prepare(const dmdh_system* s, dmd_handle* h) {
  if (!s || !h) return DMD_E_ARG;
  if (s->ee && !s->info.linear) {  // electronphonon::set_eph's e-e term (ElectronPhonon.cpp:12)
    const int rc = dmd_ee_attach(h, &s->eed);
    if (rc) return err(rc, dmd_last_error(h));
  }
  if (!s->info.ddmdteq) return dmd_set_ddmdt_eq(h, nullptr);
  // electronphonon::compute_ddmdt_eq (evolve_eph.cpp:3-19): the scattering term of diag(f_eq) at t = 0,
  // cut to the e-ph window; the stored drift is cleared first so that nothing is subtracted from it
  const dmdh_info& in = s->info;
  const int nd = in.nb_dm, nb = in.bend - in.bstart;
  const size_t nd2 = (size_t)nd * nd;
  int rc = dmd_set_ddmdt_eq(h, nullptr);
  if (rc) return err(rc, dmd_last_error(h));
  std::vector<double> y((size_t)in.nk * nd2 * 2, 0.0), y1(y.size(), 0.0), out(y.size()),
      eq((size_t)in.nk * nb * nb * 2);
  for (int ik = 0; ik < in.nk; ik++)
    for (int i = 0; i < nd; i++) {
      y[((size_t)ik * nd2 + (size_t)i * nd + i) * 2] = s->f_eq[(size_t)ik * nd + i];
      y1[((size_t)ik * nd2 + (size_t)i * nd + i) * 2] = 1 - s->f_eq[(size_t)ik * nd + i];
    }
  if (s->ee && !in.linear) {  // reset_scatt at rho_eq (DensityMatrix_Dynamics.h:58-63): P_ee(rho_eq)
    if ((rc = dmd_set_state(h, 0.0, y.data())) || (rc = dmd_ee_update(h))) return err(rc, dmd_last_error(h));
  }
  if ((rc = dmd_evolve_driver(h, 0.0, y.data(), y1.data(), out.data()))) return err(rc, dmd_last_error(h));
  for (int ik = 0; ik < in.nk; ik++)
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) {
        const size_t src = ((size_t)ik * nd2 + (size_t)(i + in.bstart) * nd + j + in.bstart) * 2;
        const size_t dst = ((size_t)ik * nb * nb + (size_t)i * nb + j) * 2;
        eq[dst] = out[src];
        eq[dst + 1] = out[src + 1];
      }
  if ((rc = dmd_set_ddmdt_eq(h, eq.data()))) return err(rc, dmd_last_error(h));
  return DMD_OK;
}

int dmdh_get_smat(const dmdh_system* s, double* smat) {
  if (!s || !smat) return DMD_E_ARG;
  memcpy(smat, s->smat.data(), s->smat.size() * 8);
  return DMD_OK;
}

int dmdh_param(const dmdh_system* s, const char* key, double unit, double* value, int* found) {
  if (!s || !key || !value || !found) return DMD_E_ARG;
  auto it = s->pm.find(key);
  *found = it != s->pm.end();
  *value = *found ? atof(it->second.c_str()) * unit : 0;
  return DMD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// DMD's time loop on the GPU (main.cpp:38-84, DensityMatrix_Dynamics.h:177-225, 322-345)
// ---------------------------------------------------------------------------------------------
namespace {

struct Reporter {
  std::string dir;
  int nv_dm, nb_dm;
  dmd_handle* h;
  int64_t freq_measure;
  bool print_tot_band;  // one more column per band of the range (the band's share of the total)
  // observable.h:169-183 (header) and 368-385 (one line per output step)
  int write_line(const std::string& what, const std::string& scarr, double t, double tot,
                 const std::vector<double>& bands, double amp) {
    const std::string fname = dir + "/" + what + scarr + "_tot.out";
    const bool fresh = !exists(fname);
    FILE* f = fopen(fname.c_str(), "a");
    if (!f) return err(DMD_E_FILE, "cannot write " + fname);
    if (fresh) fprintf(f, "#time(au), s(t), s(t) without exp(iwt)\n");
    if (fabs(t) < 1e-30) fprintf(f, " 0.00000000000000e+01 %21.14le", tot);
    else fprintf(f, "%21.14le %21.14le", t, tot);
    for (double b : bands) fprintf(f, " %21.14le", b);
    fprintf(f, " %21.14le\n", amp);
    fclose(f);
    return DMD_OK;
  }
  // the total of direction d over bands [b0, b1) and, with print_tot_band, of each band alone
  int measure_line(int d, int b0, int b1, const char* scarr, double t) {
    static const char* names[3] = {"sx", "sy", "sz"};
    double tot, amp;
    int rc;
    if ((rc = dmd_measure(h, d, b0, b1, &tot, &amp))) return err(rc, dmd_last_error(h));
    std::vector<double> bands;
    for (int i = b0; print_tot_band && i < b1; ++i) {
      double tb, ab;
      if ((rc = dmd_measure(h, d, i, i + 1, &tb, &ab))) return err(rc, dmd_last_error(h));
      bands.push_back(tb);
    }
    return write_line(names[d], scarr, t, tot, bands, amp);
  }
  int report(int it, double t, std::vector<double>& ybuf) {
    int rc;
    if (it % freq_measure != 0) return DMD_OK;  // DensityMatrix_Dynamics.h:323
    if (it > 0) {  // singdenmat_k::write_dm_tofile (DenMat.cpp:318-334), written to a temp name then renamed
      double tt;
      if ((rc = dmd_get_state(h, &tt, ybuf.data()))) return err(rc, dmd_last_error(h));
      const std::string rb = dir + "/restart/denmat_restart.bin", rt = dir + "/restart/time_restart.dat";
      FILE* fb = fopen((rb + ".tmp").c_str(), "wb");
      FILE* ft = fopen((rt + ".tmp").c_str(), "w");
      if (!fb || !ft) {
        if (fb) fclose(fb);
        if (ft) fclose(ft);
        return err(DMD_E_FILE, "cannot write restart files");
      }
      fwrite(ybuf.data(), 8, ybuf.size(), fb);
      fprintf(ft, "%14.7le", t);
      fclose(fb);
      fclose(ft);
      rename((rb + ".tmp").c_str(), rb.c_str());
      rename((rt + ".tmp").c_str(), rt.c_str());
    }
    for (int d = 0; d < 3; ++d) {
      if (nb_dm > nv_dm && (rc = measure_line(d, nv_dm, nb_dm, "_elec", t))) return rc;
      if (nv_dm > 0 && (rc = measure_line(d, 0, nv_dm, "_hole", t))) return rc;
    }
    return DMD_OK;
  }
};

const double kPs = 1000 * kFs;  // comm/Units.h

// one line of tau_<what><scarr>_tot.out (observable.h:185-191 header, 392-401 line)
int write_tau_line(const std::string& dir, const std::string& what, const std::string& scarr, double t,
                   const double tau[3], int32_t picture) {
  const std::string fname = dir + "/tau_" + what + scarr + "_tot.out";
  const bool fresh = !exists(fname);
  FILE* f = fopen(fname.c_str(), "a");
  if (!f) return err(DMD_E_FILE, "cannot write " + fname);
  if (fresh) fprintf(f, "#time(au), tau by FD, tau without precession, tau\n");
  if (picture == DMD_PICTURE_INTERACTION) {
    if (fabs(t) < 1e-30)
      fprintf(f, " 0.0000000000e+01 fs: %14.7le %14.7le %14.7le ps\n", tau[0] / kPs, tau[1] / kPs, tau[2] / kPs);
    else
      fprintf(f, "%17.10le fs: %14.7le %14.7le %14.7le ps\n", t / kFs, tau[0] / kPs, tau[1] / kPs, tau[2] / kPs);
  } else {
    if (fabs(t) < 1e-30) fprintf(f, " 0.0000000000e+01 fs: %14.7le ps\n", tau[1] / kPs);
    else fprintf(f, "%17.10le fs: %14.7le ps\n", t / kFs, tau[1] / kPs);
  }
  fclose(f);
  return DMD_OK;
}

}  // namespace

extern "C" int dmdh_tau(int32_t nk, int32_t nb, const double* obs, const double* e, const double* f,
                        const double* dm, const double* ddmdt, double t, double dt, int32_t picture, int32_t bstart,
                        int32_t bend, double prefac, double out[3]) {
  if (nk <= 0 || nb <= 0 || !obs || !e || !f || !dm || !ddmdt || !out || bstart < 0 || bend > nb || bstart >= bend)
    return DMD_E_ARG;
  const bool inter = picture == DMD_PICTURE_INTERACTION;
  const size_t nb2 = (size_t)nb * nb;
  double tot = 0, tot_tplusdt = 0, dottot = 0, dottot_term2 = 0;
  for (int ik = 0; ik < nk; ik++) {
    const zc* ok = (const zc*)obs + (size_t)ik * nb2;
    const zc* dk = (const zc*)dm + (size_t)ik * nb2;
    const zc* gk = (const zc*)ddmdt + (size_t)ik * nb2;
    const double* ek = e + (size_t)ik * nb;
    const double* fk = f + (size_t)ik * nb;
    for (int i = bstart; i < bend; i++) {
      double ob = 0, dot = 0, ob_tplusdt = 0, dot_term2 = 0;
      for (int b = 0; b < nb; b++) {
        const zc o = ok[i * nb + b];
        const zc ot = (i == b || !inter) ? o : zmul(o, zcis((ek[i] - ek[b]) * t));
        zc dkbi = dk[b * nb + i];
        if (i == b) dkbi.x = dkbi.x - fk[i];
        ob += zmul(ot, dkbi).x;
        dot += zmul(ot, gk[b * nb + i]).x;
        const zc ctmp = zmul(ot, dkbi);
        if (inter) dot_term2 -= 2 * (ctmp.y * ek[i]);
        if (dt > 0) {
          const zc otp = (i == b || !inter) ? o : zmul(o, zcis((ek[i] - ek[b]) * (t + dt)));
          zc dp = zadd(dk[b * nb + i], zscale(dt, gk[b * nb + i]));
          if (i == b) dp.x = dp.x - fk[i];
          ob_tplusdt += zmul(otp, dp).x;
        }
      }
      tot += ob;
      tot_tplusdt += ob_tplusdt;
      dottot += dot;
      dottot_term2 += dot_term2;
    }
  }
  tot *= prefac;
  tot_tplusdt *= prefac;
  dottot *= prefac;
  dottot_term2 *= prefac;
  out[0] = (dt == 0) ? 0 : -tot * dt / (tot_tplusdt - tot);
  out[1] = -tot / dottot;
  out[2] = -tot / (dottot + dottot_term2);
  return DMD_OK;
}

extern "C" int dmdh_report_tau(const dmdh_system* s, const char* dir, double t, const double* y, const double* dydt) {
  if (!s || !dir || !y || !dydt) return DMD_E_ARG;
  const dmdh_info& in = s->info;
  const int nk = in.nk, nb = in.nb_dm, nv = in.nv_dm;
  const size_t nd2 = (size_t)nb * nb;
  const double dt = std::min(in.ode_hstart, std::min(in.tstep / 10, in.tstep / 10));  // dt_tiny, tstep_laser = tstep
  const double bl = sqrt(in.Bpert[0] * in.Bpert[0] + in.Bpert[1] * in.Bpert[1] + in.Bpert[2] * in.Bpert[2]);
  const char* names[3] = {"sx", "sy", "sz"};
  std::vector<double> obs(nd2 * 2 * nk);
  for (int d = 0; d < 3; ++d) {
    if (bl > 1e-10 && in.Bpert[d] == 0) continue;  // DensityMatrix_Dynamics.h:350-352
    for (int ik = 0; ik < nk; ++ik)
      memcpy(&obs[(size_t)ik * nd2 * 2], &s->smat[((size_t)ik * 3 + d) * nd2 * 2], nd2 * 16);
    double tau[3];
    int rc;
    if (nb > nv) {
      if ((rc = dmdh_tau(nk, nb, obs.data(), s->e_dm.data(), s->f_dm.data(), y, dydt, t, dt, in.picture, nv, nb,
                         in.ob_prefac, tau)) ||
          (rc = write_tau_line(dir, names[d], "_elec", t, tau, in.picture)))
        return rc;
    }
    if (nv > 0) {
      if ((rc = dmdh_tau(nk, nb, obs.data(), s->e_dm.data(), s->f_dm.data(), y, dydt, t, dt, in.picture, 0, nv,
                         in.ob_prefac, tau)) ||
          (rc = write_tau_line(dir, names[d], "_hole", t, tau, in.picture)))
        return rc;
    }
  }
  return DMD_OK;
}

extern "C" int dmdh_run(const char* dir, int32_t precision, int64_t nsteps_max) {
  dmdh_system* s = nullptr;
  int rc = dmdh_load(dir, &s);
  if (rc) return rc;
  std::unique_ptr<dmdh_system> guard(s);
  const dmdh_info& in = s->info;
  // a new run does not overwrite the restart files of an earlier one (parameters.cpp:67-68)
  if (!s->restart && is_dir(std::string(dir) + "/restart"))
    return err(DMD_E_ARG, "directory restart presents, you should run a restart calculation");
  dmd_desc d;
  dmdh_desc(s, precision, 0, &d);
  dmd_handle* h = nullptr;
  if ((rc = dmd_create(&d, &h))) return err(rc, "dmd_create failed");
  struct Closer {
    dmd_handle* h;
    ~Closer() { dmd_destroy(h); }
  } closer{h};
  const size_t ny = (size_t)in.nk * in.nb_dm * in.nb_dm * 2;
  std::vector<double> ybuf(ny);
  if ((rc = dmdh_prepare(s, h))) return rc;
  if ((rc = dmd_set_state(h, in.t0, s->dm0.data()))) return err(rc, dmd_last_error(h));
  std::vector<double> obs((size_t)in.nk * in.nb_dm * in.nb_dm * 2);
  const size_t nd2 = (size_t)in.nb_dm * in.nb_dm;
  for (int dirn = 0; dirn < 3; ++dirn) {
    for (int ik = 0; ik < in.nk; ++ik)
      memcpy(&obs[(size_t)ik * nd2 * 2], &s->smat[((size_t)ik * 3 + dirn) * nd2 * 2], nd2 * 16);
    if ((rc = dmd_set_observable(h, dirn, obs.data(), s->f_dm.data(), in.ob_prefac))) return err(rc, dmd_last_error(h));
  }
  mkdir((std::string(dir) + "/restart").c_str(), 0755);
  Reporter rep{dir, in.nv_dm, in.nb_dm, h, s->freq_measure, s->print_tot_band != 0};
  std::vector<double> dbuf(ny);
  // compute + report_tau from the state before the step (DensityMatrix_Dynamics.h:211, 229-230):
  // the right-hand side through the GSL-callback entry, which leaves the handle's state alone
  auto tau_report = [&]() -> int {
    double tt;
    int r;
    if ((r = dmd_get_state(h, &tt, ybuf.data())) || (r = dmd_func(h, tt, ybuf.data(), dbuf.data())))
      return err(r, dmd_last_error(h));
    return dmdh_report_tau(s, dir, tt, ybuf.data(), dbuf.data());
  };
  // the initial excess quantities (a restart continues the files of the earlier run), then with
  // compute_tau_only the lifetimes at t0 and no evolution (DensityMatrix_Dynamics.h:72-75, main.cpp:79)
  if (!s->restart && (rc = rep.report(0, in.t0, ybuf))) return rc;
  if (s->compute_tau_only) return tau_report();
  double t = in.t0, ti = in.t0, hs = in.ode_hstart;
  const std::string stopfile = std::string(dir) + "/EXIT_DMD";
  for (int64_t it = 1; t < in.tend && (nsteps_max < 0 || it <= nsteps_max); ++it) {
    if (exists(stopfile)) {  // "touch EXIT_DMD" clean exit (DensityMatrix_Dynamics.h:244)
      remove(stopfile.c_str());
      break;
    }
    const bool tau_now = (it - 1) % s->freq_compute_tau == 0;
    if (tau_now && in.ode_method != 1 && (rc = tau_report())) return rc;  // evolve_gsl: before the update
    ti += in.tstep;
    // update_scatt_outside (DensityMatrix_Dynamics.h:216-217, 290-299): the e-e operators from the
    // state before every freq_update_ee_model-th step
    if (s->ee_freq > 0 && (it - 1) % s->ee_freq == 0 && (rc = dmd_ee_update(h))) return err(rc, dmd_last_error(h));
    if (tau_now && in.ode_method == 1 && (rc = tau_report())) return rc;  // evolve_euler: after it
    int64_t nfev = 0;
    if (in.ode_method == 0) rc = dmd_rkf45_apply(h, ti, &hs, in.ode_hmin, in.ode_hmax, in.ode_epsabs, 0.0, &nfev);
    else if (in.ode_method == 1) rc = dmd_euler(h, in.tstep, 1), nfev = 1;
    else rc = dmd_rk4(h, in.tstep, 1), nfev = 4;
    if (rc) return err(rc, dmd_last_error(h));
    if ((rc = dmd_get_state(h, &t, nullptr))) return err(rc, dmd_last_error(h));
    if ((rc = rep.report((int)it, t, ybuf))) return rc;
    printf("ncalls= %lld at ti= %lg fs\n", (long long)nfev, ti / kFs);
    fflush(stdout);
  }
  return DMD_OK;
}
