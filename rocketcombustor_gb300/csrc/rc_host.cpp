// Host side of the RocketCombustor steady solver for callers without the
// Fortran host: case-file readers and the reference's one-time set-up, in the
// module-array layout that rc_init takes (see include/rc_host.h).
//
// Arithmetic follows the reference expressions term by term; this file is
// compiled with -ffp-contract=off so that no a*b+c is fused into an FMA.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "rc_host.h"
#include "rc_math.h"

namespace {

// ------------------------------------------------------- record reader -----
// Fortran list-directed input: a READ starts on a fresh record, takes values
// separated by blanks or commas across records and drops the rest of its last
// record; a READ with an empty list skips one record.
class Records {
 public:
  explicit Records(const std::string& path) : path_(path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    text_ = ss.str();
  }
  void skip() {
    size_t e = text_.find('\n', pos_);
    pos_ = (e == std::string::npos) ? text_.size() : e + 1;
  }
  std::vector<std::string> take(size_t n) {
    std::vector<std::string> v;
    while (v.size() < n) {
      if (pos_ >= text_.size()) throw std::runtime_error("unexpected end of " + path_);
      size_t e = line_end();
      for (size_t p = pos_; p < e && v.size() < n;) {
        while (p < e && sep(text_[p])) ++p;
        size_t q = p;
        while (q < e && !sep(text_[q])) ++q;
        if (q > p) v.emplace_back(text_, p, q - p);
        p = q;
      }
      pos_ = e + 1;
    }
    return v;
  }
  // All integers of the next record (one cell record: kface n1 .. nk).
  int record_ints(long* out, int maxn) {
    if (pos_ >= text_.size()) throw std::runtime_error("unexpected end of " + path_);
    size_t e = line_end();
    int k = 0;
    const char* s = text_.c_str();
    for (size_t p = pos_; p < e && k < maxn;) {
      while (p < e && sep(text_[p])) ++p;
      if (p >= e) break;
      char* q;
      out[k++] = std::strtol(s + p, &q, 10);
      p = (size_t)(q - s);
    }
    pos_ = e + 1;
    return k;
  }
  // n numbers spanning as many records as needed.
  void numbers(size_t n, std::vector<double>& out) {
    out.resize(n);
    size_t k = 0;
    const char* s = text_.c_str();
    while (k < n) {
      if (pos_ >= text_.size()) throw std::runtime_error("unexpected end of " + path_);
      size_t e = line_end();
      for (size_t p = pos_; p < e && k < n;) {
        while (p < e && sep(text_[p])) ++p;
        if (p >= e) break;
        char* q;
        out[k++] = std::strtod(s + p, &q);
        p = (size_t)(q - s);
      }
      pos_ = e + 1;
    }
  }
  double real() { return std::strtod(take(1)[0].c_str(), nullptr); }
  long integer() { return std::strtol(take(1)[0].c_str(), nullptr, 10); }
  static bool logical(const std::string& s) {
    for (char c : s)
      if (c != '.') return c == 't' || c == 'T';
    return false;
  }

 private:
  static bool sep(char c) { return c == ' ' || c == ',' || c == '\t' || c == '\r'; }
  size_t line_end() const {
    size_t e = text_.find('\n', pos_);
    return e == std::string::npos ? text_.size() : e;
  }
  std::string path_, text_;
  size_t pos_ = 0;
};

double num(const std::string& s) { return std::strtod(s.c_str(), nullptr); }
long inum(const std::string& s) { return std::strtol(s.c_str(), nullptr, 10); }
double fmax2(double a, double b) { return (b > a) ? b : a; }

// Thirteen-point triangle rule (gaussInteg4.f90:4-42) of integrand f.
template <class F>
double tri_rule(const double* a, const double* b, const double* c, F f) {
  const double area = 0.5 * std::fabs((b[0] - a[0]) * (c[1] - a[1]) - (c[0] - a[0]) * (b[1] - a[1]));
  double p[13][2];
  for (int d = 0; d < 2; ++d) p[0][d] = (a[d] + b[d] + c[d]) / 3.0;
  const double A[3] = {0.479308067841920, 0.869739794195568, 0.048690315425316};
  const double B[3] = {0.260345966079040, 0.065130102902216, 0.312865496004874};
  for (int s = 0; s < 2; ++s)
    for (int d = 0; d < 2; ++d) {
      p[1 + 3 * s][d] = A[s] * a[d] + B[s] * (b[d] + c[d]);
      p[2 + 3 * s][d] = A[s] * b[d] + B[s] * (a[d] + c[d]);
      p[3 + 3 * s][d] = A[s] * c[d] + B[s] * (a[d] + b[d]);
    }
  const double al = A[2], be = B[2], ga = 1 - al - be;
  for (int d = 0; d < 2; ++d) {
    p[7][d] = al * a[d] + be * b[d] + ga * c[d];
    p[8][d] = al * a[d] + be * c[d] + ga * b[d];
    p[9][d] = al * b[d] + be * a[d] + ga * c[d];
    p[10][d] = al * b[d] + be * c[d] + ga * a[d];
    p[11][d] = al * c[d] + be * a[d] + ga * b[d];
    p[12][d] = al * c[d] + be * b[d] + ga * a[d];
  }
  const double g = -0.149570044467682 * f(p[0]) + 0.175615257433208 * (f(p[1]) + f(p[2]) + f(p[3])) +
                   0.053347235608838 * (f(p[4]) + f(p[5]) + f(p[6])) +
                   0.077113760890257 * (f(p[7]) + f(p[8]) + f(p[9]) + f(p[10]) + f(p[11]) + f(p[12]));
  return g * area;
}
// GaussInteg_Quad (gaussInteg4.f90:44-50): triangles (1,2,3) and (1,3,4).
template <class F>
double quad_rule(const double* const* v, F f) {
  return tri_rule(v[0], v[1], v[2], f) + tri_rule(v[0], v[2], v[3], f);
}

}  // namespace

// ------------------------------------------------------------- the case ----
struct rc_case {
  std::string dir, err;
  int Nsp = 0, NVar = 0, model = 0;
  double Rconstant = 0;
  std::vector<double> mw, Rsp, cl, ch, b1l, b1h, muK[16], sigma, eps, cf, cr;
  double tlo = 0, tcr = 0, thi = 0, trlo = 0, trcr = 0, trhi = 0, Af = 0, E = 0;
  std::vector<double> oxY, fuY;
  double oxT = 0, oxP = 0, oxM = 0, fuT = 0, fuP = 0, fuM = 0;
  bool combustion = false, viscous = false, backup = false;
  int limit = 0, nscreen = 1;
  long nstep = 0;
  double unit = 1, cfl = 0, p_out_ratio = 0, p_out = 0;
  // unsteady dual-time BDF2 (implicit_time_method 5)
  bool steady = true;
  int inner_loop = 1, method = 5;
  double totaltime = 0, rel_tol = 0, A_p = 0, f_p = 0, p_static = 0, ttime = 0, dt = 0;
  // module arrays, Fortran layout, 1-based ids
  int NE = 0, NF = 0, NNT = 0, MaxNei = 0, Ng = 0;
  std::vector<int> KFace, N, Neighbor, FNode, FProperty, NeighF, Neigh, NeighC, Ghostcell, Num_ghostcell,
      Hostcell, Hostface, BCtype;
  std::vector<double> COOR, VECX, SideOfs, VOL, CELLXY, reflen, wdis, AMLS, CoorG, CxyG, volG, XYH;
  double total_volume = 0;
  std::vector<double> PA, WA;

  const double* xy(int node) const { return &COOR[2 * (size_t)(node - 1)]; }
  int& Nk(int k, int i) { return N[(size_t)(k - 1) + 4 * (size_t)(i - 1)]; }
  int& Nb(int s, int f) { return Neighbor[(size_t)(s - 1) + 2 * (size_t)(f - 1)]; }

  void read_inputs();
  void read_mesh();
  void initialise();
  void stencils();
  void gas(const double* Y, double T, double& Cp, double& gama, double& R) const;
  void enthalpy(double T, double* h) const;
};

void rc_case::read_inputs() {
  const std::string c = dir + "/combustion/";
  {  // setup_species_info (species.f90:14-51)
    Records r(c + "species.in");
    r.skip();
    Nsp = (int)r.integer();
    if (Nsp < 1) throw std::runtime_error("Nsp < 1");
    r.skip();
    mw.resize(Nsp);
    for (int i = 0; i < Nsp; ++i) mw[i] = num(r.take(2)[1]);
    r.skip();
    Rconstant = r.real();
    Rsp.resize(Nsp);
    for (int i = 0; i < Nsp; ++i) Rsp[i] = Rconstant / mw[i];
    NVar = 4 + Nsp - 1;  // setup_number_of_variables (species.f90:53-65)
  }
  {  // setup_thermo_property (thermo_property.f90:18-59)
    Records r(c + "thermo.in");
    r.skip(); r.real();
    r.skip();
    if (r.integer() != 7) throw std::runtime_error("order_of_cp_polynomial must be 7");
    r.skip();
    auto t = r.take(3);
    tlo = num(t[0]); tcr = num(t[1]); thi = num(t[2]);
    cl.assign(7 * (size_t)Nsp, 0); ch.assign(7 * (size_t)Nsp, 0);
    b1l.assign(Nsp, 0); b1h.assign(Nsp, 0);
    for (int i = 0; i < Nsp; ++i) {
      auto a = r.take(7);
      for (int j = 0; j < 7; ++j) cl[j + 7 * (size_t)i] = num(a[j]);
      b1l[i] = r.real();
      auto b = r.take(7);
      for (int j = 0; j < 7; ++j) ch[j + 7 * (size_t)i] = num(b[j]);
      b1h[i] = r.real();
    }
  }
  {  // setup_transport_property (transport_property.f90:16-48)
    Records r(c + "transport.in");
    r.skip();
    auto t = r.take(3);
    trlo = num(t[0]); trcr = num(t[1]); trhi = num(t[2]);
    r.skip();
    for (auto& v : muK) v.assign(Nsp, 0);
    for (int i = 0; i < Nsp; ++i)
      for (int row = 0; row < 4; ++row) {
        auto v = r.take(4);
        for (int k = 0; k < 4; ++k) muK[row * 4 + k][i] = num(v[k]);
      }
  }
  {  // setup_diffusion_velocity (diffusion_velocity.f90:15-41)
    Records r(c + "diffusion.in");
    r.skip(); r.real(); r.skip();
    sigma.resize(Nsp); eps.resize(Nsp);
    for (int i = 0; i < Nsp; ++i) {
      auto v = r.take(2);
      sigma[i] = num(v[0]); eps[i] = num(v[1]);
    }
  }
  {  // setup_chemical_kinetics (chemical_kinetics.f90:16-57); the rate models use reaction 1
    Records r(c + "chemical_kinetics.in");
    r.skip();
    auto v = r.take(2);
    long nreact = inum(v[0]);
    model = (int)inum(v[1]);
    if (nreact < 1) throw std::runtime_error("need at least one reaction");
    if (model != 0 && model != 1) throw std::runtime_error("No such code_chemical_model");
    r.skip();
    cf.resize(Nsp); cr.resize(Nsp);
    for (long q = 0; q < nreact; ++q)
      for (int j = 0; j < Nsp; ++j) {
        auto s = r.take(2);
        if (q == 0) { cf[j] = num(s[0]); cr[j] = num(s[1]); }
      }
    r.skip();
    for (long q = 0; q < nreact; ++q) {
      auto s = r.take(3);
      if (q == 0) { Af = num(s[0]); E = num(s[2]); }
    }
  }
  auto inlet = [&](const char* f, std::vector<double>& Y, double& T, double& p, double& m) {
    Records r(c + f);  // oxidizer.f90:13-41, fuel.f90:13-41
    r.skip();
    Y.resize(Nsp);
    for (int i = 0; i < Nsp; ++i) Y[i] = r.real();
    r.skip();
    auto v = r.take(2);
    T = num(v[0]); p = num(v[1]);
    r.skip();
    m = r.real();
  };
  inlet("oxidizer.in", oxY, oxT, oxP, oxM);
  inlet("fuel.in", fuY, fuT, fuP, fuM);
  {  // startup.f90:55-128
    Records r(dir + "/flow/flow_solver_info.in");
    r.skip(); combustion = Records::logical(r.take(1)[0]);
    r.skip(); bool right = Records::logical(r.take(1)[0]);
    r.skip(); r.integer();
    r.skip(); long npar = r.integer();
    r.skip(); unit = r.real();
    r.skip();
    auto f = r.take(4);
    steady = Records::logical(f[0]);
    viscous = Records::logical(f[1]);
    backup = Records::logical(f[2]);
    bool expl = Records::logical(f[3]);
    r.skip(); method = (int)r.integer();
    r.skip();
    auto g = r.take(5);
    cfl = num(g[0]);
    totaltime = num(g[1]);
    nstep = inum(g[2]);
    r.skip(); r.take(1);
    r.skip();
    auto il = r.take(3);
    inner_loop = (int)inum(il[1]);
    rel_tol = num(il[2]);
    r.skip(); nscreen = (int)inum(r.take(4)[0]);
    r.skip(); r.real();
    r.skip(); limit = (int)inum(r.take(2)[1]);
    r.skip();
    long nmon = r.integer();
    r.skip();
    for (long i = 0; i < nmon; ++i) r.take(2);
    r.skip();
    auto po = r.take(3);
    p_out_ratio = num(po[0]);
    A_p = num(po[1]);
    f_p = num(po[2]);
    if (expl || right || npar != 1 || (!steady && method != 5 && method != 3))
      throw std::runtime_error(
          "the GPU path covers the steady implicit and the unsteady BDF2 / backward Euler single-partition solver");
    if (steady) inner_loop = 1;                    // initParam.f90:64-66
    else dt = totaltime / (double)nstep;           // initParam.f90:72
  }
}

// ReadMesh (mesh.f90:2-115) with change/face (:120-199) and VolumeAndCenter (:206-286).
void rc_case::read_mesh() {
  Records r(dir + "/grid1.in");
  auto h = r.take(6);
  long v[6];
  for (int k = 0; k < 6; ++k) v[k] = inum(h[k]);
  if (v[0] != v[1] || v[2] != v[3] || v[4] != v[5]) throw std::runtime_error("single-partition meshes only");
  NE = (int)v[0]; NNT = (int)v[2]; NF = (int)v[4];
  KFace.assign(NE, 0);
  N.assign(4 * (size_t)NE, 0);
  long rec[8];
  for (int i = 1; i <= NE; ++i) {
    int n = r.record_ints(rec, 8);
    int kf = (int)rec[0];
    if (kf < 3 || kf > 4 || n < kf + 1) throw std::runtime_error("bad cell record");
    KFace[i - 1] = kf;
    for (int k = 1; k <= kf; ++k) Nk(k, i) = (int)rec[k];
    if (kf == 3) Nk(4, i) = Nk(3, i);
  }
  MaxNei = *std::max_element(KFace.begin(), KFace.end());
  std::vector<double> c4;
  r.numbers(4 * (size_t)NNT, c4);
  COOR.resize(2 * (size_t)NNT);
  for (int p = 0; p < NNT; ++p) { COOR[2 * p] = c4[4 * p] / unit; COOR[2 * p + 1] = c4[4 * p + 1] / unit; }
  if (r.integer() != 0) throw std::runtime_error("NConE must be 0 on one partition");
  auto nbh = r.take(2);
  int nbound = (int)inum(nbh[0]);
  // first boundary group listing an edge gives its type (mesh.f90:76-93)
  std::unordered_map<uint64_t, int> btype;
  auto key = [](long a, long b) { return ((uint64_t)std::min(a, b) << 32) | (uint64_t)std::max(a, b); };
  for (int ib = 0; ib < nbound; ++ib) {
    auto t = r.take(2);
    int itype = (int)inum(t[0]);
    long nbf = inum(t[1]);
    std::vector<double> pr;
    r.numbers(2 * (size_t)nbf, pr);
    for (long q = 0; q < nbf; ++q) btype.emplace(key((long)pr[2 * q], (long)pr[2 * q + 1]), itype);
  }
  if (r.integer() != 0) throw std::runtime_error("periodic pairs (NCon>0) are not supported");
  // faces in the order cells first meet them (change/face)
  Neighbor.assign(2 * (size_t)NF, -100);
  FNode.assign(2 * (size_t)NF, 0);
  VECX.assign(2 * (size_t)NF, 0.0);
  SideOfs.assign(2 * (size_t)NF, 0.0);
  FProperty.assign(NF, 0);
  std::unordered_map<uint64_t, int> edge;
  edge.reserve((size_t)NF * 2);
  int nfc = 0;
  for (int j = 1; j <= NE; ++j) {
    const int kf = KFace[j - 1];
    for (int k = 1; k <= kf; ++k) {
      const int n1 = Nk(k, j), n2 = Nk(k % kf + 1, j);
      auto it = edge.find(key(n1, n2));
      if (it == edge.end()) {
        if (nfc >= NF) throw std::runtime_error("error in number of face");
        ++nfc;
        edge.emplace(key(n1, n2), nfc);
        Nb(1, nfc) = j;
        VECX[2 * (size_t)(nfc - 1)] = xy(n2)[1] - xy(n1)[1];
        VECX[2 * (size_t)(nfc - 1) + 1] = -(xy(n2)[0] - xy(n1)[0]);
        FNode[2 * (size_t)(nfc - 1)] = n1;
        FNode[2 * (size_t)(nfc - 1) + 1] = n2;
      } else {
        Nb(2, it->second) = j;
      }
    }
  }
  if (nfc != NF) throw std::runtime_error("error in number of face");
  for (int f = 1; f <= NF; ++f)
    if (Nb(2, f) < 0) {
      auto it = btype.find(key(FNode[2 * (size_t)(f - 1)], FNode[2 * (size_t)(f - 1) + 1]));
      if (it == btype.end()) throw std::runtime_error("not find boundary of this type");
      Nb(2, f) = -it->second;
    }
  // VolumeAndCenter
  VOL.assign(NE, 0); CELLXY.assign(2 * (size_t)NE, 0); reflen.assign(2 * (size_t)NE, 0);
  for (int i = 1; i <= NE; ++i) {
    const double* v4[4] = {xy(Nk(1, i)), xy(Nk(2, i)), xy(Nk(3, i)), xy(Nk(4, i))};
    const double vol = quad_rule(v4, [](const double*) { return 1.0; });
    VOL[i - 1] = vol;
    CELLXY[2 * (size_t)(i - 1)] = quad_rule(v4, [](const double* q) { return q[0]; }) / vol;
    CELLXY[2 * (size_t)(i - 1) + 1] = quad_rule(v4, [](const double* q) { return q[1]; }) / vol;
    if (vol < 0.0) throw std::runtime_error("negative volume");
    double* rl = &reflen[2 * (size_t)(i - 1)];
    for (int a = 1; a < KFace[i - 1]; ++a)
      for (int b = a + 1; b <= KFace[i - 1]; ++b)
        for (int d = 0; d < 2; ++d) rl[d] = fmax2(0.5 * std::fabs(xy(Nk(a, i))[d] - xy(Nk(b, i))[d]), rl[d]);
  }
  double s = 0.0;
  for (int i = 0; i < NE; ++i) s = s + VOL[i];
  total_volume = s;
}

// ComputeGasParameter (thermo_property.f90:78-112), host copy.
void rc_case::gas(const double* Y, double T, double& Cp, double& gama, double& R) const {
  const double t2 = T * T;
  const double b[7] = {1.0 / t2, 1.0 / T, 1.0, T, t2, T * t2, t2 * t2};
  const bool low = (tlo <= T && T <= tcr);
  if (!low && !(tcr < T && T <= thi)) throw std::runtime_error("temperature out of the thermo range");
  const std::vector<double>& c = low ? cl : ch;
  double cp = 0.0, r = 0.0;
  std::vector<double> cps(Nsp);
  for (int i = 0; i < Nsp; ++i) {
    double s = 0.0;
    for (int j = 0; j < 7; ++j) s = s + c[j + 7 * (size_t)i] * b[j];
    cps[i] = s * Rsp[i];
  }
  for (int i = 0; i < Nsp; ++i) cp = cp + cps[i] * Y[i];
  for (int i = 0; i < Nsp; ++i) r = r + Rsp[i] * Y[i];
  Cp = cp; R = r; gama = cp / (cp - r);
}
// compute_enthalpy (thermo_property.f90:114-144), host copy.
void rc_case::enthalpy(double T, double* h) const {
  const double t2 = T * T;
  const double e[7] = {-(1.0 / t2), rcm::log(T) / T, 1.0, T / 2.0, t2 / 3.0, (T * t2) / 4.0, (t2 * t2) / 5.0};
  const bool low = (tlo <= T && T <= tcr);
  if (!low && !(tcr < T && T <= thi)) throw std::runtime_error("temperature out of the thermo range");
  const std::vector<double>& c = low ? cl : ch;
  for (int i = 0; i < Nsp; ++i) {
    double s = 0.0;
    for (int j = 0; j < 7; ++j) s = s + c[j + 7 * (size_t)i] * e[j];
    h[i] = Rsp[i] * (T * s + (low ? b1l[i] : b1h[i]));
  }
}

// initialization (initialization.f90:17-35 + 156-201) and Read_Backup
// (output.f90:276-338) followed by primitve_to_conserved_variables
// (update_flow_variables.f90:50-84).  The reference fills hard-coded
// combustor zones first (:70-146), which the backup then overwrites; those
// zones assume four species and are left out.
void rc_case::initialise() {
  double min_ox = 1.0e10, max_ox = -1.0e10, min_fu = 1.0e10, max_fu = -1.0e10;
  for (int f = 0; f < NF; ++f) {
    const double y1 = xy(FNode[2 * f])[1], y2 = xy(FNode[2 * f + 1])[1];
    const double lo = (y2 < y1) ? y2 : y1, hi = (y2 > y1) ? y2 : y1;
    if (Neighbor[2 * f + 1] == -3) { min_ox = (lo < min_ox) ? lo : min_ox; max_ox = fmax2(hi, max_ox); }
    if (Neighbor[2 * f + 1] == -4) { min_fu = (lo < min_fu) ? lo : min_fu; max_fu = fmax2(hi, max_fu); }
  }
  const double ox_d = 2 * (max_ox - min_ox), fu_d = max_fu - min_fu;
  oxM = oxM / ox_d;
  fuM = 0.5 * fuM / fu_d;
  p_out = p_out_ratio * oxP;
  p_static = p_out;
  if (!backup) throw std::runtime_error("the initial field is read from fvp1.sav (IfReadBackup=.true.)");
  Records r(dir + "/fvp1.sav");
  ttime = r.real();
  if (r.integer() != NE) throw std::runtime_error("Error in the number of cells when reading backup");
  std::vector<double> row;
  PA.assign((size_t)NVar * NE, 0);
  WA.assign((size_t)NVar * NE, 0);
  for (int i = 0; i < NE; ++i) {
    r.numbers(2 + (size_t)NVar, row);
    for (int k = 0; k < NVar; ++k) PA[(size_t)i * NVar + k] = row[2 + k];
  }
  std::vector<double> Y(Nsp), h(Nsp);
  for (int i = 0; i < NE; ++i) {
    const double* P = &PA[(size_t)i * NVar];
    double s = 0.0;
    for (int k = 0; k < Nsp - 1; ++k) { Y[k] = P[4 + k]; s = s + Y[k]; }
    Y[Nsp - 1] = 1.0 - s;
    double Cp, gama, R;
    gas(Y.data(), P[3], Cp, gama, R);
    const double rr = P[0] / (R * P[3]);
    enthalpy(P[3], h.data());
    double hh = 0.0;
    for (int k = 0; k < Nsp; ++k) hh = hh + Y[k] * h[k];
    double* W = &WA[(size_t)i * NVar];
    W[0] = rr;
    W[1] = rr * P[1];
    W[2] = rr * P[2];
    W[3] = rr * (hh + 0.5 * (P[1] * P[1] + P[2] * P[2])) - P[0];
    for (int k = 0; k < Nsp - 1; ++k) W[4 + k] = rr * Y[k];
  }
}

// compute_reconstruction_matrix (reconstruction_initialization.f90:1-167) with
// construct_ghostcells (ghostcell.f90:19-181).  The LAPACK pseudo-inverse
// (la_math.f90:1-62) of the full-rank kface x 2 matrix is taken in closed
// form, (A^T A)^-1 A^T.
void rc_case::stencils() {
  const int M = MaxNei;
  NeighF.assign(4 * (size_t)NE, 0);
  std::vector<int> cnt(NE, 0);
  for (int f = 1; f <= NF; ++f) {
    const int L = Nb(1, f), R = Nb(2, f);
    NeighF[4 * (size_t)(L - 1) + cnt[L - 1]++] = f;
    if (R > 0) NeighF[4 * (size_t)(R - 1) + cnt[R - 1]++] = f;
  }
  Neigh.assign(NE, 0);
  NeighC.assign((size_t)(M + 1) * NE, 0);
  for (int i = 1; i <= NE; ++i) {
    int* nc = &NeighC[(size_t)(M + 1) * (i - 1)];
    nc[0] = i;
    for (int k = 0; k < KFace[i - 1]; ++k) {
      const int f = NeighF[4 * (size_t)(i - 1) + k];
      for (int s = 1; s <= 2; ++s) {
        const int c = Nb(s, f);
        if (c != i && c > 0) nc[++Neigh[i - 1]] = c;
      }
    }
  }
  // ghost cells: a mirrored cell behind every boundary face of a cell
  Ng = 0;
  for (int i = 0; i < NE; ++i) Ng += KFace[i] - Neigh[i];
  Hostcell.assign(Ng, 0); Hostface.assign(Ng, 0); BCtype.assign(Ng, 0);
  Ghostcell.assign((size_t)M * NE, 0); Num_ghostcell.assign(NE, 0);
  CoorG.assign(8 * (size_t)Ng, 0); CxyG.assign(2 * (size_t)Ng, 0); volG.assign(Ng, 0);
  int j = 0;
  for (int i = 1; i <= NE; ++i) {
    const int kf = KFace[i - 1];
    for (int q = 0; q < kf && Neigh[i - 1] < kf; ++q) {
      const int f = NeighF[4 * (size_t)(i - 1) + q];
      if (Nb(2, f) >= 0) continue;
      ++j;
      Hostcell[j - 1] = i;
      Hostface[j - 1] = f;
      BCtype[j - 1] = -Nb(2, f);
      Ghostcell[(size_t)M * (i - 1) + Num_ghostcell[i - 1]++] = j;
      const int n1 = FNode[2 * (size_t)(f - 1)], n2 = FNode[2 * (size_t)(f - 1) + 1];
      int k1 = 1;
      while (k1 <= kf && Nk(k1, i) != n1) ++k1;
      const int k2 = k1 % kf + 1;
      if (k1 > kf || Nk(k2, i) != n2) throw std::runtime_error("error in index setting of nodes of a ghost cell");
      const int k3 = k2 % kf + 1, k4 = k3 % kf + 1;
      const int n3 = Nk(k3, i), n4 = Nk(k4, i);
      const double sav1 = VECX[2 * (size_t)(f - 1)], sav2 = VECX[2 * (size_t)(f - 1) + 1];
      const double sav = fmax2(std::sqrt(sav1 * sav1 + sav2 * sav2), 1.0e-16);
      const double s1 = sav1 / sav, s2 = sav2 / sav;
      double* g = &CoorG[8 * (size_t)(j - 1)];
      g[0] = xy(n2)[0]; g[1] = xy(n2)[1];
      g[2] = xy(n1)[0]; g[3] = xy(n1)[1];
      const double d1 = (xy(n1)[0] - xy(n4)[0]) * s1 + (xy(n1)[1] - xy(n4)[1]) * s2;
      if (d1 < 0) throw std::runtime_error("error in calculating the distance of a ghost node (n1,n4)");
      g[4] = xy(n4)[0] + 2 * d1 * s1; g[5] = xy(n4)[1] + 2 * d1 * s2;
      const double d2 = (xy(n2)[0] - xy(n3)[0]) * s1 + (xy(n2)[1] - xy(n3)[1]) * s2;
      if (d2 < 0) throw std::runtime_error("error in calculating the distance of a ghost node (n2,n3)");
      g[6] = xy(n3)[0] + 2 * d2 * s1; g[7] = xy(n3)[1] + 2 * d2 * s2;
      const double* v4[4] = {g, g + 2, g + 4, g + 6};
      const double vol = quad_rule(v4, [](const double*) { return 1.0; });
      volG[j - 1] = vol;
      CxyG[2 * (size_t)(j - 1)] = quad_rule(v4, [](const double* p) { return p[0]; }) / vol;
      CxyG[2 * (size_t)(j - 1) + 1] = quad_rule(v4, [](const double* p) { return p[1]; }) / vol;
      if (vol < 0.0) throw std::runtime_error("negative ghost volume");
    }
    if (Num_ghostcell[i - 1] + Neigh[i - 1] != kf) throw std::runtime_error("error in number of ghost cells");
  }
  // first moments of the scaled coordinates (must vanish)
  XYH.assign(2 * (size_t)NE, 0);
  for (int i = 1; i <= NE; ++i) {
    const double cx = CELLXY[2 * (size_t)(i - 1)], cy = CELLXY[2 * (size_t)(i - 1) + 1];
    const double lx = reflen[2 * (size_t)(i - 1)], ly = reflen[2 * (size_t)(i - 1) + 1];
    const double* v4[4] = {xy(Nk(1, i)), xy(Nk(2, i)), xy(Nk(3, i)), xy(Nk(4, i))};
    XYH[2 * (size_t)(i - 1)] = quad_rule(v4, [&](const double* p) { return (p[0] - cx) / lx; }) / VOL[i - 1];
    XYH[2 * (size_t)(i - 1) + 1] = quad_rule(v4, [&](const double* p) { return (p[1] - cy) / ly; }) / VOL[i - 1];
    if (std::fabs(XYH[2 * (size_t)(i - 1)]) + std::fabs(XYH[2 * (size_t)(i - 1) + 1]) > 1.e-8)
      throw std::runtime_error("error in XYH");
  }
  wdis.assign((size_t)M * NE, 1.0);
  AMLS.assign(2 * (size_t)M * NE, 0.0);
  std::vector<double> A;
  for (int i = 1; i <= NE; ++i) {
    const int kf = KFace[i - 1], nn = Neigh[i - 1];
    const double cx = CELLXY[2 * (size_t)(i - 1)], cy = CELLXY[2 * (size_t)(i - 1) + 1];
    const double lx = reflen[2 * (size_t)(i - 1)], ly = reflen[2 * (size_t)(i - 1) + 1];
    const double h1 = XYH[2 * (size_t)(i - 1)], h2 = XYH[2 * (size_t)(i - 1) + 1];
    A.assign(2 * (size_t)kf, 0.0);
    double* w = &wdis[(size_t)M * (i - 1)];
    for (int k = 1; k <= nn; ++k) {
      const int c = NeighC[(size_t)(M + 1) * (i - 1) + k];
      // SideOfs is zero without periodic pairs: x - 0 == x
      const double* v4[4] = {xy(Nk(1, c)), xy(Nk(2, c)), xy(Nk(3, c)), xy(Nk(4, c))};
      const double dx = CELLXY[2 * (size_t)(c - 1)] - 0.0 - cx, dy = CELLXY[2 * (size_t)(c - 1) + 1] - 0.0 - cy;
      w[k - 1] = 1.0 / std::sqrt(dx * dx + dy * dy);
      A[k - 1] = w[k - 1] * (quad_rule(v4, [&](const double* p) { return (p[0] - cx) / lx; }) / VOL[c - 1] - h1);
      A[kf + k - 1] = w[k - 1] * (quad_rule(v4, [&](const double* p) { return (p[1] - cy) / ly; }) / VOL[c - 1] - h2);
    }
    for (int k = 1; k <= Num_ghostcell[i - 1]; ++k) {
      const int g = Ghostcell[(size_t)M * (i - 1) + k - 1];
      const double* G = &CoorG[8 * (size_t)(g - 1)];
      const double* v4[4] = {G, G + 2, G + 4, G + 6};
      const double dx = CxyG[2 * (size_t)(g - 1)] - cx, dy = CxyG[2 * (size_t)(g - 1) + 1] - cy;
      const int m = k + nn;
      w[m - 1] = 1.0 / std::sqrt(dx * dx + dy * dy);
      A[m - 1] = w[m - 1] * (quad_rule(v4, [&](const double* p) { return (p[0] - cx) / lx; }) / volG[g - 1] - h1);
      A[kf + m - 1] = w[m - 1] * (quad_rule(v4, [&](const double* p) { return (p[1] - cy) / ly; }) / volG[g - 1] - h2);
    }
    double g11 = 0.0, g12 = 0.0, g22 = 0.0;
    for (int k = 0; k < kf; ++k) {
      g11 = g11 + A[k] * A[k];
      g12 = g12 + A[k] * A[kf + k];
      g22 = g22 + A[kf + k] * A[kf + k];
    }
    const double det = g11 * g22 - g12 * g12;
    double* am = &AMLS[2 * (size_t)M * (i - 1)];
    for (int k = 0; k < kf; ++k) {
      am[2 * k] = (g22 * A[k] - g12 * A[kf + k]) / det;
      am[2 * k + 1] = (g11 * A[kf + k] - g12 * A[k]) / det;
    }
  }
}

// ------------------------------------------------------------ C ABI -------
static std::string g_case_error;

extern "C" {

int rc_case_open(const char* case_dir, rc_case** out) {
  *out = nullptr;
  auto* c = new rc_case();
  try {
    c->dir = case_dir;
    c->read_inputs();
    c->read_mesh();
    c->initialise();
    c->stencils();
  } catch (const std::exception& e) {
    g_case_error = e.what();
    delete c;
    return RC_ERR_ARG;
  }
  *out = c;
  return RC_OK;
}

const char* rc_case_error(const rc_case* c) { return c ? c->err.c_str() : g_case_error.c_str(); }
void rc_case_close(rc_case* c) { delete c; }

int rc_case_views(rc_case* c, int precision, int device, rc_mesh* m, rc_thermo* t, rc_config* g) {
  if (!c || !m || !t || !g) return RC_ERR_ARG;
  m->NE = c->NE; m->NF = c->NF; m->NNT = c->NNT; m->MaxNei = c->MaxNei; m->Nghostcell = c->Ng;
  m->KFace = c->KFace.data(); m->Neighbor = c->Neighbor.data(); m->FNode = c->FNode.data();
  m->FProperty = c->FProperty.data(); m->NeighF = c->NeighF.data(); m->Neigh = c->Neigh.data();
  m->NeighC = c->NeighC.data(); m->Ghostcell = c->Ghostcell.data(); m->Num_ghostcell = c->Num_ghostcell.data();
  m->Hostcell = c->Hostcell.data(); m->BCtype_Ghostcell = c->BCtype.data();
  m->COOR = c->COOR.data(); m->VECX = c->VECX.data(); m->SideOfs = c->SideOfs.data(); m->VOL = c->VOL.data();
  m->CELLXY = c->CELLXY.data(); m->reflen = c->reflen.data(); m->wdis = c->wdis.data(); m->AMLS = c->AMLS.data();
  m->Coor_Ghostnode = c->CoorG.data(); m->total_volume = c->total_volume;
  t->Nsp = c->Nsp; t->Rconstant = c->Rconstant; t->mole_weight = c->mw.data(); t->R_species = c->Rsp.data();
  t->order_of_cp_polynomial = 7;
  t->thermo_lowest_tem = c->tlo; t->thermo_critical_tem = c->tcr; t->thermo_highest_tem = c->thi;
  t->low_coef_Cp_species = c->cl.data(); t->high_coef_Cp_species = c->ch.data();
  t->low_enthalpy_b1 = c->b1l.data(); t->high_enthalpy_b1 = c->b1h.data();
  t->transport_lowest_tem = c->trlo; t->transport_critical_tem = c->trcr; t->transport_highest_tem = c->trhi;
  for (int k = 0; k < 16; ++k) t->mu_K[k] = c->muK[k].data();
  t->collision_diameter = c->sigma.data(); t->LJ_energy = c->eps.data();
  t->code_chemical_model = c->model; t->coef_f_react = c->cf.data(); t->coef_r_react = c->cr.data();
  t->Af_react = c->Af; t->E_react = c->E;
  t->oxidizer_mass_fraction = c->oxY.data(); t->oxidizer_temp_in = c->oxT; t->oxidizer_mass_flow = c->oxM;
  t->fuel_mass_fraction = c->fuY.data(); t->fuel_temp_in = c->fuT; t->fuel_mass_flow = c->fuM;
  g->IfViscous = c->viscous; g->If_turn_on_combustion = c->combustion; g->limit_ID = c->limit;
  g->cfl = c->cfl; g->p_out = c->p_out; g->precision = precision; g->device = device;
  return RC_OK;
}

void rc_case_dims(const rc_case* c, long* d) {
  d[0] = c->NE; d[1] = c->NF; d[2] = c->NNT; d[3] = c->NVar; d[4] = c->Nsp; d[5] = c->MaxNei; d[6] = c->Ng;
  d[7] = c->nstep; d[8] = c->nscreen;
}
const double* rc_case_PA(const rc_case* c) { return c->PA.data(); }
const double* rc_case_WA(const rc_case* c) { return c->WA.data(); }

const void* rc_case_array(const rc_case* c, const char* name, long* count) {
  const std::string s(name);
#define RC_ARR(nm, v)                 \
  if (s == nm) {                      \
    *count = (long)c->v.size();       \
    return (const void*)c->v.data();  \
  }
  RC_ARR("KFace", KFace) RC_ARR("N", N) RC_ARR("Neighbor", Neighbor) RC_ARR("FNode", FNode)
  RC_ARR("FProperty", FProperty) RC_ARR("NeighF", NeighF) RC_ARR("Neigh", Neigh) RC_ARR("NeighC", NeighC)
  RC_ARR("Ghostcell", Ghostcell) RC_ARR("Num_ghostcell", Num_ghostcell) RC_ARR("Hostcell", Hostcell)
  RC_ARR("Hostface", Hostface) RC_ARR("BCtype_Ghostcell", BCtype) RC_ARR("COOR", COOR) RC_ARR("VECX", VECX)
  RC_ARR("SideOfs", SideOfs) RC_ARR("VOL", VOL) RC_ARR("CELLXY", CELLXY) RC_ARR("reflen", reflen)
  RC_ARR("wdis", wdis) RC_ARR("AMLS", AMLS) RC_ARR("Coor_Ghostnode", CoorG) RC_ARR("CellXY_Ghostcell", CxyG)
  RC_ARR("vol_Ghostcell", volG) RC_ARR("XYH", XYH) RC_ARR("PA", PA) RC_ARR("WA", WA)
#undef RC_ARR
  *count = 0;
  return nullptr;
}

int rc_case_set_state(rc_case* c, const double* PA, const double* WA) {
  if (!c || !PA || !WA) return RC_ERR_ARG;
  std::copy(PA, PA + (size_t)c->NVar * c->NE, c->PA.begin());
  std::copy(WA, WA + (size_t)c->NVar * c->NE, c->WA.begin());
  return RC_OK;
}

// BackupData (output.f90:256-273): ttime, NE, then per cell x, y, PA(1:NVar).
// List-directed in the reference; written here with 17 significant digits so
// that Read_Backup (output.f90:276-338) restores the state bit for bit.
int rc_case_write_backup(rc_case* c, const char* path, double ttime) {
  if (!c || !path) return RC_ERR_ARG;
  std::FILE* f = std::fopen(path, "w");
  if (!f) { c->err = std::string("cannot write ") + path; return RC_ERR_ARG; }
  std::fprintf(f, " %.17E\n %d\n", ttime, c->NE);
  for (int i = 0; i < c->NE; ++i) {
    std::fprintf(f, " %.17E %.17E", c->CELLXY[2 * (size_t)i], c->CELLXY[2 * (size_t)i + 1]);
    for (int k = 0; k < c->NVar; ++k) std::fprintf(f, " %.17E", c->PA[(size_t)i * c->NVar + k]);
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  if (!ok) { c->err = std::string("cannot write ") + path; return RC_ERR_ARG; }
  return RC_OK;
}

namespace {
// Fortran Ew.d edit descriptor: 0.d1d2..dd E+xx (leading zero, d digits)
std::string fortran_e(double x, int d, int w) {
  char m[64];
  std::string out;
  if (x == 0.0 || !std::isfinite(x)) {
    std::snprintf(m, sizeof m, "%.*f", d, 0.0);
    out = std::isfinite(x) ? std::string(m) + "E+00" : (x != x ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
  } else {
    int e = (int)std::floor(std::log10(std::fabs(x))) + 1;
    double mant = x / std::pow(10.0, e);
    if (std::fabs(mant) >= 1.0) { mant /= 10.0; ++e; }
    if (std::fabs(mant) < 0.1) { mant *= 10.0; --e; }
    std::snprintf(m, sizeof m, "%.*f", d, mant);
    if (std::fabs(std::atof(m)) >= 1.0) { mant /= 10.0; ++e; std::snprintf(m, sizeof m, "%.*f", d, mant); }
    char ex[16];
    std::snprintf(ex, sizeof ex, "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
    out = std::string(m) + ex;
  }
  if ((int)out.size() < w) out = std::string((size_t)w - out.size(), ' ') + out;
  return out;
}
std::string ltrim(const std::string& s) {
  const size_t a = s.find_first_not_of(' ');
  return a == std::string::npos ? std::string() : s.substr(a);
}
}  // namespace

// output_vtk (output.f90:5-227): legacy ASCII VTK of the cell-centred rho, u,
// v, p, T, Ma, Y_1..Y_Nsp and the production rates of the transported species
// (compute_production_rate, chemical_kinetics.f90:109-165, at the state; the
// reference writes its module copy from the last sourceterm).  Values below
// 1e-15 are written as 0 as in the reference (output.f90:51-54).
int rc_case_write_vtk(rc_case* c, const char* path) {
  if (!c || !path) return RC_ERR_ARG;
  const int NE = c->NE, Nsp = c->Nsp, NVar = c->NVar;
  std::vector<double> rho(NE), ma(NE), Y((size_t)Nsp * NE), prod((size_t)Nsp * NE, 0.0);
  std::vector<double> y(Nsp), w(Nsp);
  try {
    for (int i = 0; i < NE; ++i) {
      const double* P = &c->PA[(size_t)i * NVar];
      double s = 0.0;
      for (int k = 0; k < Nsp - 1; ++k) { y[k] = P[4 + k]; s = s + y[k]; }
      y[Nsp - 1] = 1.0 - s;
      double Cp, gama, R;
      c->gas(y.data(), P[3], Cp, gama, R);
      rho[i] = P[0] / (R * P[3]);
      const double ac = std::sqrt(gama * R * P[3]);
      ma[i] = std::sqrt(P[1] * P[1] + P[2] * P[2]) / ac;
      if (P[0] < 0 || rho[i] < 0 || P[3] < 0) {
        c->err = "negative density/pressure/temperature in cell " + std::to_string(i + 1);
        return RC_ERR_NEG_TIMESTEP;
      }
      if (c->combustion && Nsp > 1) {  // compute_production_rate, model 0 or 1
        const double y0 = std::min(1.0, std::max(0.0, y[0])), y1 = std::min(1.0, std::max(0.0, y[1]));
        double kf;
        if (c->model == 0) {
          kf = c->Af * rcm::exp(-c->E / (c->Rconstant * P[3]));
          kf = kf * rcm::pow(y0 * rho[i] / (c->mw[0] * 1000), 0.2);
          kf = kf * rcm::pow(y1 * rho[i] / (c->mw[1] * 1000), 1.3);
        } else {
          kf = (P[3] > 710.0) ? 1e4 : 0.0;
          kf = kf * (y0 * rho[i] / (c->mw[0] * 1000));
        }
        for (int k = 0; k < Nsp; ++k) w[k] = 1000 * c->mw[k] * (c->cr[k] - c->cf[k]) * kf;
        if (std::fabs(w[0]) < 1.0e-15)
          for (int k = 0; k < Nsp; ++k) w[k] = 0.0;
        for (int k = 0; k < Nsp; ++k) prod[(size_t)k * NE + i] = w[k];
      }
      for (int k = 0; k < Nsp; ++k) {
        double v = y[k];
        if (k < Nsp - 1 && std::fabs(v) < 1.0e-15) v = 0.0;
        Y[(size_t)k * NE + i] = v;
      }
    }
  } catch (const std::exception& e) {
    c->err = e.what();
    return RC_ERR_THERMO_T;
  }
  std::FILE* f = std::fopen(path, "w");
  if (!f) { c->err = std::string("cannot write ") + path; return RC_ERR_ARG; }
  std::fprintf(f, "# vtk DataFile Version 1.0\nUnstructured Grid Format\nASCII\nDATASET UNSTRUCTURED_GRID\n");
  std::fprintf(f, "POINTS %d double\n", c->NNT);
  for (int n = 0; n < c->NNT; ++n)
    std::fprintf(f, "%s\n", ltrim(fortran_e(c->COOR[2 * (size_t)n], 8, 15) + fortran_e(c->COOR[2 * (size_t)n + 1], 8, 15) +
                                   fortran_e(0.0, 8, 15)).c_str());
  long nsize = NE;
  for (int i = 0; i < NE; ++i) nsize += c->KFace[i];
  std::fprintf(f, "CELLS %d %ld\n", NE, nsize);
  for (int i = 0; i < NE; ++i) {
    std::fprintf(f, "%d", c->KFace[i]);
    for (int k = 0; k < c->KFace[i]; ++k) std::fprintf(f, " %d", c->N[(size_t)k + 4 * (size_t)i] - 1);
    std::fputc('\n', f);
  }
  std::fprintf(f, "CELL_TYPES %d\n", NE);
  for (int i = 0; i < NE; ++i) std::fprintf(f, "%d\n", c->KFace[i] == 3 ? 5 : 9);
  std::fprintf(f, "CELL_DATA %d\n", NE);
  auto scalars = [&](const char* name, const double* v, size_t stride, int d, int wdt) {
    std::fprintf(f, "SCALARS %s double\nLOOKUP_TABLE default\n", name);
    for (int i = 0; i < NE; ++i) std::fprintf(f, "%s\n", ltrim(fortran_e(v[(size_t)i * stride], d, wdt)).c_str());
  };
  std::vector<double> col(NE);
  scalars("rho", rho.data(), 1, 8, 20);
  for (int q = 0; q < 4; ++q) {
    for (int i = 0; i < NE; ++i) col[i] = c->PA[(size_t)i * NVar + (q == 0 ? 1 : q == 1 ? 2 : q == 2 ? 0 : 3)];
    scalars(q == 0 ? "u" : q == 1 ? "v" : q == 2 ? "p" : "T", col.data(), 1, 8, 20);
  }
  scalars("Ma", ma.data(), 1, 8, 20);
  for (int k = 0; k < Nsp; ++k) {
    const std::string nm = "Y" + std::to_string(k + 1);
    scalars(nm.c_str(), &Y[(size_t)k * NE], 1, 12, 30);
  }
  for (int k = 0; k < Nsp - 1; ++k) {
    const std::string nm = "Production_rate_" + std::to_string(k + 1);
    scalars(nm.c_str(), &prod[(size_t)k * NE], 1, 12, 30);
  }
  const bool ok = std::fclose(f) == 0;
  if (!ok) { c->err = std::string("cannot write ") + path; return RC_ERR_ARG; }
  return RC_OK;
}

int rc_run_steady(rc_case* c, int precision, int device, long nsteps, long every, double* hist) {
  rc_mesh m;
  rc_thermo t;
  rc_config g;
  rc_case_views(c, precision, device, &m, &t, &g);
  rc_ctx* ctx = nullptr;
  int st = rc_init(&m, &t, &g, &ctx);
  if (st) { c->err = "rc_init failed"; return st; }
  st = rc_set_state(ctx, c->PA.data(), c->WA.data());
  long row = 0;
  for (long it = 1; it <= nsteps && !st; ++it) {
    st = rc_lusgs_stage(ctx, (int)it);
    if (!st && hist && every > 0 && it % every == 0) {
      st = rc_residual(ctx, hist + (size_t)row * (c->NVar + 1), hist + (size_t)row * (c->NVar + 1) + c->NVar);
      ++row;
    }
  }
  if (!st) st = rc_get_state(ctx, c->PA.data(), c->WA.data());
  if (st) c->err = rc_last_error(ctx);
  rc_finalize(ctx);
  return st;
}

int rc_case_unsteady(const rc_case* c, double* out) {
  if (!c || !out) return RC_ERR_ARG;
  out[0] = c->steady ? 0.0 : 1.0; out[1] = c->ttime; out[2] = c->dt; out[3] = c->totaltime;
  out[4] = (double)c->nstep; out[5] = c->inner_loop; out[6] = c->rel_tol; out[7] = c->p_static;
  out[8] = c->A_p; out[9] = c->f_p; out[10] = c->method;
  return RC_OK;
}

// compute_p_out (fvm2d.f90:229-239)
static double case_p_out(const rc_case* c, double ttime) {
  const double pi = 4 * std::atan(1.0);
  return c->p_static * (1. + c->A_p * std::sin(2 * pi * c->f_p * ttime));
}

// The unsteady implicit branch of program main (fvm2d.f90:48-150) with the
// BDF2 or backward Euler stage (implicit_time_method 5 or 3): per physical step the last step is shortened to end at
// totaltime (:52-56), ttime and p_out advance around the stage, and the loop
// ends after that last step.
int rc_run_unsteady(rc_case* c, int device, long nsteps, long every, double* hist, int* inner) {
  if (!c || nsteps < 0 || (hist && every < 1)) return RC_ERR_ARG;
  if (c->steady) { c->err = "the case is steady (IfSteady = .true.)"; return RC_ERR_ARG; }
  rc_mesh m;
  rc_thermo t;
  rc_config g;
  rc_case_views(c, RC_PREC_FP64, device, &m, &t, &g);
  rc_ctx* ctx = nullptr;
  int st = rc_init(&m, &t, &g, &ctx);
  if (st) { c->err = "rc_init failed"; return st; }
  st = rc_set_state(ctx, c->PA.data(), c->WA.data());
  const double totaltime_num = c->totaltime * (1. - 1.e-10);
  long row = 0;
  for (long istep = 1; istep <= nsteps && !st; ++istep) {
    bool stop = false;
    if (c->ttime + c->dt > totaltime_num) { c->dt = c->totaltime - c->ttime; stop = true; }
    const double ttime_n = c->ttime;
    c->ttime = ttime_n + 1.0 * c->dt;
    c->p_out = case_p_out(c, c->ttime);
    st = rc_set_p_out(ctx, &c->p_out);
    int n_inner = 0;
    if (!st)
      st = c->method == 3 ? rc_euler_stage(ctx, (int)istep, c->dt, c->inner_loop, c->rel_tol, &n_inner)
                          : rc_bdf2_stage(ctx, (int)istep, c->dt, c->inner_loop, c->rel_tol, &n_inner);
    if (inner) inner[istep - 1] = n_inner;
    c->ttime = ttime_n + c->dt;
    c->p_out = case_p_out(c, c->ttime);
    if (!st && hist && istep % every == 0) {
      st = rc_residual(ctx, hist + (size_t)row * (c->NVar + 1), hist + (size_t)row * (c->NVar + 1) + c->NVar);
      ++row;
    }
    if (stop) break;
  }
  if (!st) st = rc_get_state(ctx, c->PA.data(), c->WA.data());
  if (st) c->err = rc_last_error(ctx);
  rc_finalize(ctx);
  return st;
}

// Mixed precision with defect correction: iterate in RC_PREC_MIXED and switch
// once to RC_PREC_MIXED_DC (FP64 residual, FP32 sweeps) when the FP32
// residual stalls: at every residual check r = max_k Res_k / Res_k(first
// check) over the non-zero columns; a check that does not bring r below 0.99
// times its best value so far counts towards the stall, `window` such checks
// in a row switch.  switched_at gets the iteration of the switch (0: none).
int rc_run_steady_dc(rc_case* c, int device, long nsteps, long every, int window, double* hist, long* switched_at) {
  if (!c || every < 1 || window < 1) return RC_ERR_ARG;
  rc_mesh m;
  rc_thermo t;
  rc_config g;
  rc_case_views(c, RC_PREC_MIXED_DC, device, &m, &t, &g);
  rc_ctx* ctx = nullptr;
  int st = rc_init(&m, &t, &g, &ctx);
  if (st) { c->err = "rc_init failed"; return st; }
  st = rc_set_precision(ctx, RC_PREC_MIXED);
  if (!st) st = rc_set_state(ctx, c->PA.data(), c->WA.data());
  const int V = c->NVar;
  std::vector<double> res(V), res0;
  double best = 1e300, romax = 0.0;
  int since = 0;
  long row = 0, sw = 0;
  for (long it = 1; it <= nsteps && !st; ++it) {
    st = rc_lusgs_stage(ctx, (int)it);
    if (st || it % every) continue;
    st = rc_residual(ctx, res.data(), &romax);
    if (st) break;
    if (hist) {
      for (int k = 0; k < V; ++k) hist[(size_t)row * (V + 1) + k] = res[k];
      hist[(size_t)row * (V + 1) + V] = romax;
    }
    ++row;
    if (res0.empty()) res0 = res;
    double r = 0.0;
    for (int k = 0; k < V; ++k)
      if (res0[k] > 0.0) r = std::max(r, res[k] / res0[k]);
    if (sw) continue;
    if (r < 0.99 * best) {
      best = r;
      since = 0;
    } else if (++since >= window) {
      st = rc_set_precision(ctx, RC_PREC_MIXED_DC);
      sw = it;
    }
  }
  if (switched_at) *switched_at = sw;
  if (!st) st = rc_get_state(ctx, c->PA.data(), c->WA.data());
  if (st) c->err = rc_last_error(ctx);
  rc_finalize(ctx);
  return st;
}

}  // extern "C"
