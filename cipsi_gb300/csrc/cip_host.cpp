// cip_host.cpp -- host side of the GPU drop-in for cip.exe / cipsym.exe.
//
// Reads what the reference reads (namelists &cipfil and &icinp on standard
// input; units 40 ijkl, 33 ener, 60 det, 59 bdvec, 4 f04), builds the
// reference space with its spin-flip partners, computes the zero-order
// quantities, hands everything to the engine through the C ABI of
// cipsi_gb300.h, and writes what the reference writes after the perturbation
// (unit 60 with S and the selected perturbers, unit 33 energy records, the
// listing lines the Autocip driver parses).
//
// Followed sources: cip/cip.f:50-254 and 403-425 (main flow, outputs),
// cip/openf.f, cip/deter.f:78-251 and 478-567, cip/transf.f, cip/lec60.f,
// cip/ijkf.f, cip/reijkl.f, cip/rdener.f, cip/ic001.f:44-76, cip/faifoc.f,
// cip/hmp.f, cip/hdig.f, cip/pie.f, cip/stkener.f and the cipsym variants
// (cipsym/cip.f:226-254, cipsym/pie.f, cipsym/ic001.f:179).
//
// Supported: the perturbation run with lecdet 5 (S from unit 60, vectors
// from unit 59) or with lecdet 2, 3, 4 (S from unit 60 or a complete active
// space, diagonalised here on the GPU as cip/ic001.f:81-131 does); and the
// run that only writes S (ityper < 0,
// cip/cip.f:200-236), with S from unit 60 (lecdet 2, 3, 5) or generated as
// a complete active space (lecdet 4, cip/cas.f) -- the two ways the Autocip
// driver calls cipsym (Autocip_13/calcul.f90:318-353).  isz = 0.  Other
// inputs are rejected with a message.

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/cipsi_gb300.h"
#include "host_io.h"

namespace {

using namespace cipsi_host;


struct Options {
  // &icinp (defaults of cip/deter.f:78-226)
  double test = 0.5, teseff = -1.0, tau = 1.0e-4, tdet = 0.0, coeff = 0.0;
  int isz = 0, metat = 1, ityper = 1, iselec = 1, lecdet = 1, nclass = 10, maxdet = 500000;
  int ninact = 0;
  bool yion = false, ybrd = false, ymoyen = false, ywdeg = true, ytocom = false;
  int ydp = -1;  // -1: as the unit-40 header says; 0/1: set in &icinp
  double aval[10] = {0.128e-6, 0.64e-6, 0.32e-5, 0.16e-4, 0.8e-4, 0.4e-3, 0.2e-2, 0.1e-1, 0.5e-1, 1.0};
  std::string title = "                    ";
  std::map<int, double> tocom;  // elements assigned in &icinp (1-based)
  std::map<int, int> numero;    // state numbers (default 1..metat)
  // complete active space of lecdet = 4 (COMMON /activ/, cip/cas.f); cip's
  // cas.f has no nemax (cipsym/cas.f:227)
  int noac = 0, nelac = 0, nusym = 1, nemax = 8;
  bool use_nemax = true;
  std::map<int, int> numac;  // active orbitals (default 1..norb)
  // &cipfil
  std::string f60 = "det", f40 = "ijkl", f04 = "f04", f59 = "bdvec", f33 = "ener", f21 = "ocno";
};

// the names of the namelists (cip/openf.f:5-6, cip/deter.f:52-57; cipsym's
// &icinp adds nemax, cipsym/deter.f:58)
const std::set<std::string> kCipfilNames = {"prefix", "det",   "ijkl",  "f04",   "det1",  "ijkl1", "f041",
                                            "ocno1",  "bdvec", "bdvec1", "ocno", "ener", "ener1"};
const std::set<std::string> kIcinpNames = {
    "test",  "ndiag", "isz",    "metat",  "tocom", "yprt",   "yion",   "ybrd",   "ityper", "numero",
    "coeff", "ygen",  "title",  "tau",    "ymoyen", "aval",  "nclass", "ytoul",  "lecdet", "tdet",
    "maxdet", "teseff", "nvr",  "numac",  "nelac", "nusym",  "noac",   "ywvi",   "ywvf",   "ystkic",
    "ywdeg", "ytocom", "iselec", "iord",  "twdet", "mspin",  "ydp",    "ninact", "nonact"};


Options read_options(const std::string& text, const std::string& dir, bool sym_variant) {
  Options o;
  Namelist cf = parse_namelist(text, "cipfil", kCipfilNames);
  o.f60 = unit_file(cf, "det", "det1", "det", dir);
  o.f40 = unit_file(cf, "ijkl", "ijkl1", "ijkl", dir);
  o.f04 = unit_file(cf, "f04", "f041", "f04", dir);
  o.f59 = unit_file(cf, "bdvec", "bdvec1", "bdvec", dir);
  o.f33 = unit_file(cf, "ener", "ener1", "ener", dir);
  o.f21 = unit_file(cf, "ocno", "ocno1", "ocno", dir);
  std::set<std::string> names = kIcinpNames;
  if (sym_variant) names.insert("nemax");
  o.use_nemax = sym_variant;
  Namelist ic = parse_namelist(text, "icinp", names);
  if (!ic.found) throw Error("erreur dans la namelist icinp");
  auto r1 = [&](const char* k, double& d) { if (auto v = ic.scalar(k)) d = to_real(*v); };
  auto i1 = [&](const char* k, int& d) { if (auto v = ic.scalar(k)) d = to_int(*v); };
  auto l1 = [&](const char* k, bool& d) { if (auto v = ic.scalar(k)) d = to_logical(*v); };
  r1("test", o.test); r1("teseff", o.teseff); r1("tau", o.tau); r1("tdet", o.tdet); r1("coeff", o.coeff);
  i1("isz", o.isz); i1("metat", o.metat); i1("ityper", o.ityper); i1("iselec", o.iselec);
  i1("lecdet", o.lecdet); i1("nclass", o.nclass); i1("maxdet", o.maxdet); i1("ninact", o.ninact);
  i1("noac", o.noac); i1("nelac", o.nelac); i1("nusym", o.nusym);
  if (sym_variant) i1("nemax", o.nemax);
  l1("yion", o.yion); l1("ybrd", o.ybrd); l1("ymoyen", o.ymoyen); l1("ywdeg", o.ywdeg); l1("ytocom", o.ytocom);
  if (const std::string* v = ic.scalar("ydp")) o.ydp = to_logical(*v);
  for (auto& e : ic.array("numac", 512)) o.numac[e.first] = to_int(e.second);
  for (auto& e : ic.array("aval", 10)) o.aval[e.first - 1] = to_real(e.second);
  for (auto& e : ic.array("tocom", 512)) o.tocom[e.first] = to_real(e.second);
  for (auto& e : ic.array("numero", 60)) o.numero[e.first] = to_int(e.second);
  (void)ic.array("nonact", 512);
  (void)ic.array("mspin", 60);
  if (const std::string* v = ic.scalar("title")) {
    o.title = *v;
    o.title.resize(20, ' ');
  }
  if (ic.has("ygen")) throw Error("ygen given in &icinp is not supported");
  if (ic.has("iord")) throw Error("iord given in &icinp is not supported");
  if (o.lecdet == 5) o.tdet = 0.0;  // deter.f:224-226: the whole of unit 60
  return o;
}

// numero(m+1): the number printed and stored for root m (default m+1)
int state_number(const Options& o, int m) {
  const auto it = o.numero.find(m + 1);
  return it != o.numero.end() ? it->second : m + 1;
}

// ------------------------------------------------------------ the run state
struct Space {
  std::vector<int32_t> ne, nd, trou, part;
  std::vector<uint8_t> ygen, ysaut, yef1;
  std::vector<int32_t> nesp;
  std::set<std::vector<int>> keys;  // sorted lists of every determinant (transf.f:76-85)
  bool insert(int nec, const int* t, const int* p) {
    std::vector<int> key(t, t + nec);
    key.insert(key.end(), p, p + nec);
    return keys.insert(std::move(key)).second;
  }
};

struct Run {
  Options o;
  int nsym = 1, norb = 0, noc = 0, isym = 0, ncf = 0, metat = 1;
  bool ydp = true;
  std::vector<int32_t> itsym, its;  // its column-major nsym x nsym
  std::vector<double> F, J, K;
  std::vector<int16_t> ij0;
  std::vector<int32_t> ntttt;
  std::vector<float> eri;
  double escf = 0.0;
  Space S;
  std::vector<double> c, e, eb, emp, teste, taum, fmpb, fdiag;
  std::vector<double> tocom, empdet;  // faifoc.f occupations (after cip.f:75-84), hmp of S
  std::vector<double> hdiag;          // hdig of S
  std::vector<double> tocom21;        // occupations read from unit 21 (ytocom)
  int device = -1;  // the GPU of the S diagonalisation (lecdet != 5); -1: none allowed
};

// transf.f: sort, validate, dedup and append one determinant
void transf(Run& R, int nec, int* nt, int* np) {
  const int norb = R.norb, mnorb = 2 * norb, noca = R.noc, nocb = R.noc + norb;
  if (nec == 0) {
    if (!R.S.insert(0, nullptr, nullptr)) return;
    R.S.ne.push_back(0);
    R.S.nd.push_back((int)R.S.trou.size());
    R.isym = 1;
    return;
  }
  std::sort(nt, nt + nec);
  std::sort(np, np + nec);
  int is = 1, ls = 0;
  auto bad = [&](const char* m) { throw Error(std::string(m)); };
  if (nt[0] < 1 || np[nec - 1] > mnorb || nt[nec - 1] > nocb || np[nec - 1] <= noca)
    bad("1 spin orbitale est hors de l espace de base");
  for (int i = 0; i < nec; ++i) {
    if (!(nt[i] <= noca) && nt[i] < norb + 1) bad("1 spin orbitale est hors de l espace de base");
    if (!(np[i] > nocb)) {
      if (np[i] > norb) bad("1 spin orbitale est hors de l espace de base");
      if (np[i] <= noca) bad("1 spin orbitale est hors de l espace de base");
    }
    const int st = R.itsym[(nt[i] - 1) % norb], sp = R.itsym[(np[i] - 1) % norb];
    is = R.its[(size_t)(st - 1) * R.nsym + (is - 1)];
    is = R.its[(size_t)(sp - 1) * R.nsym + (is - 1)];
    ls += (np[i] > norb) - (nt[i] > norb);
  }
  if (R.isym == 0) R.isym = is;
  if (is != R.isym) bad("dterminant de mauvaise symetrie");
  if (ls != 0) bad("mauvais spin");
  if (!R.S.insert(nec, nt, np)) return;
  R.S.ne.push_back(nec);
  R.S.nd.push_back((int)R.S.trou.size());
  for (int j = 0; j < nec; ++j) {
    R.S.trou.push_back(nt[j]);
    R.S.part.push_back(np[j]);
  }
}

// The determinants of S before the spin-flip closure: whether the reference
// determinant is there, and the others by excitation degree (holes then
// particles, in the order in which deter.f:478-567 appends them).
struct DetLists {
  bool hf = false;
  std::vector<std::vector<std::vector<int>>> byrank = std::vector<std::vector<std::vector<int>>>(9);
};

// lec60.f: the determinants of unit 60 with v >= tdet
DetLists read_unit60(const Run& R, const std::string& f60) {
  DetLists L;
  auto& byrank = L.byrank;
  bool& hf = L.hf;
  int ndet = 0;
  for (auto& rec : read_records(f60)) {
    const int mw = rec.get<int32_t>(), nw = rec.get<int32_t>();
    std::vector<int32_t> idet(mw), nex(nw);
    std::vector<double> v(nw);
    for (auto& x : idet) x = rec.get<int32_t>();
    for (auto& x : nex) x = rec.get<int32_t>();
    for (auto& x : v) x = rec.get<double>();
    int my = 0;
    for (int l = 0; l < nw; ++l) {
      const int nec = nex[l];
      if (nec > 8 || nec < 0) throw Error("erreur degre d excitation depasse les possibilites du programme");
      if (v[l] < R.o.tdet) {
        my += 2 * nec;
        continue;
      }
      if (++ndet > R.o.maxdet) {
        if (R.o.lecdet == 3) goto done;
        throw Error("trop de determinants selectionnes sur la file60");
      }
      std::vector<int> d(2 * nec);
      for (int s = 0; s < nec; ++s) {
        d[s] = idet[my++];
        d[s + nec] = idet[my++];
      }
      if (nec == 0)
        hf = true;
      else
        byrank[nec].push_back(std::move(d));
    }
  }
done:
  return L;
}

// cas.f: the complete active space of lecdet = 4.  Each spin has
// n = (nelac+1)/2 electrons in the active orbitals numac[0..noac), of which
// the first n are the ones the reference determinant occupies.  A spin string
// is an increasing n-tuple of active positions, enumerated in lexicographic
// order, and becomes the holes it leaves among the first n positions and the
// particles it puts among the others (as orbital numbers, in position order).
// Determinants run over alpha strings (outer loop) and beta strings (inner);
// those with more than nemax excitations or a symmetry other than nusym (the
// first determinant's when nusym = 0) are skipped.  Limits and messages are
// the reference's: 20 active electrons, 25000 strings of one spin, 500000
// determinants, 10 holes + particles per string.
DetLists cas_space(Run& R) {
  Options& o = R.o;
  DetLists L;
  if (o.nelac > 20) throw Error(" trop d electrons actifs  maximum 20");
  const int n = (o.nelac + 1) / 2, noac = o.noac;
  if (n > noac) throw Error("more active electrons of one spin than active orbitals (nelac, noac)");
  if (n == 0) return L;  // no beta string: no determinant (cas.f:188-200)
  std::vector<int> act(noac);
  for (int k = 0; k < noac; ++k) {
    const auto it = o.numac.find(k + 1);
    act[k] = it != o.numac.end() ? it->second : k + 1;  // deter.f:139 default numac(i) = i
    if (act[k] < 1 || act[k] > R.norb) throw Error("numac names an orbital outside 1..norb");
  }
  struct Str {
    std::vector<int> t, p;
  };
  std::vector<Str> strs;
  std::vector<int> pos(n);
  for (int i = 0; i < n; ++i) pos[i] = i;
  for (;;) {
    if ((int)strs.size() >= 25000) throw Error("  trop de combinaisons: max=25000");
    std::vector<bool> in(noac, false);
    for (int q : pos) in[q] = true;
    Str st;
    for (int k = 0; k < n; ++k)
      if (!in[k]) st.t.push_back(act[k]);
    for (int k = n; k < noac; ++k)
      if (in[k]) st.p.push_back(act[k]);
    if (st.t.size() + st.p.size() > 10) throw Error("more than 10 holes and particles in one CAS string");
    strs.push_back(std::move(st));
    int i = n - 1;  // lexicographic successor of pos
    while (i >= 0 && pos[i] == noac - n + i) --i;
    if (i < 0) break;
    ++pos[i];
    for (int k = i + 1; k < n; ++k) pos[k] = pos[k - 1] + 1;
  }
  const int norb = R.norb, nsym = R.nsym;
  auto prod = [&](int a, int b) { return R.its[(size_t)(b - 1) * nsym + (a - 1)]; };
  int ndet = 0;
  for (const Str& a : strs)
    for (const Str& b : strs) {
      std::vector<int> t(a.t), p(a.p);
      for (int x : b.t) t.push_back(x + norb);
      for (int x : b.p) p.push_back(x + norb);
      const int nec = (int)t.size();
      if (o.use_nemax && nec > o.nemax) continue;
      int is = 1;
      for (int i = 0; i < nec; ++i) {
        is = prod(is, R.itsym[(t[i] - 1) % norb]);
        is = prod(is, R.itsym[(p[i] - 1) % norb]);
      }
      if (o.nusym == 0) o.nusym = is;
      if (is != o.nusym) continue;
      if (++ndet > 500000) throw Error(" espace actif trop grand  maximum=500000");
      if (nec == 0) {
        L.hf = true;
        continue;
      }
      if (nec > 8) throw Error("CAS determinant with more than 8 excitations (nemax > 8)");
      std::vector<int> d(t);
      d.insert(d.end(), p.begin(), p.end());
      L.byrank[nec].push_back(std::move(d));
    }
  return L;
}

// deter.f:478-567: S from the lists, each determinant followed by its
// spin-flip partner
void build_space(Run& R, const DetLists& L) {
  const auto& byrank = L.byrank;
  if (L.hf) transf(R, 0, nullptr, nullptr);
  R.S.ygen.assign(R.S.ne.size(), 0);
  R.S.ysaut.assign(R.S.ne.size(), 0);
  R.S.yef1.assign(R.S.ne.size(), 0);
  R.S.nesp.assign(R.S.ne.size(), 0);
  const int norb = R.norb;
  auto flip = [&](int so) { return so <= norb ? so + norb : so - norb; };
  for (int nec = 1; nec <= 8; ++nec)
    for (auto& d : byrank[nec]) {
      const size_t before = R.S.ne.size();
      int nt[8], np[8];
      for (int l = 0; l < nec; ++l) {
        nt[l] = d[l];
        np[l] = d[l + nec];
      }
      transf(R, nec, nt, np);
      if (R.S.ne.size() == before) continue;
      R.S.ygen.push_back(0);
      R.S.ysaut.push_back(0);
      R.S.yef1.push_back(0);
      R.S.nesp.push_back(0);
      int ft[8], fp[8];
      for (int l = 0; l < nec; ++l) {
        ft[l] = flip(nt[l]);
        fp[l] = flip(np[l]);
      }
      transf(R, nec, ft, fp);
      if (R.S.ne.size() > before + 1) {
        R.S.ygen.push_back(0);
        R.S.ysaut.push_back(1);
        R.S.yef1.push_back(1);
        R.S.nesp.push_back(0);
        R.S.yef1[before] = 1;
        R.S.nesp[before] = 1;
      }
    }
  R.ncf = (int)R.S.ne.size();
  if (R.ncf == 0) throw Error("erreur dans les donnees: aucun determinant dans le sous espace variationnel");
}

// hmp / hdig of an S determinant from its excitation lists (cip/hmp.f, hdig.f)
double hmp_list(const Run& R, int k) {
  double ac = 0.0;
  for (int l = 0; l < R.S.ne[k]; ++l) ac = ac + R.fmpb[R.S.part[R.S.nd[k] + l] - 1] - R.fmpb[R.S.trou[R.S.nd[k] + l] - 1];
  return ac;
}

double hdig_list(const Run& R, int k) {
  const int n = R.norb;
  auto num = [](int i) { return i * (i - 1) / 2; };
  double ab = 0.0;
  const int l1 = R.S.nd[k], nei = R.S.ne[k];
  for (int l = 0; l < nei; ++l) {
    int n1p = R.S.part[l1 + l], n1t = R.S.trou[l1 + l];
    ab = ab + R.fdiag[n1p - 1] - R.fdiag[n1t - 1];
    const int ns1t = n1t > n, ns1p = n1p > n;
    n1t = (n1t - 1) % n + 1;
    n1p = (n1p - 1) % n + 1;
    for (int j = 0; j <= l; ++j) {
      int n2t = R.S.trou[l1 + j], n2p = R.S.part[l1 + j];
      const int ns2t = n2t > n, ns2p = n2p > n;
      n2t = (n2t - 1) % n + 1;
      n2p = (n2p - 1) % n + 1;
      const int n12t = n2t > n1t ? num(n2t) + n1t : num(n1t) + n2t;
      const int n12p = n2p > n1p ? num(n2p) + n1p : num(n1p) + n2p;
      const int n1tp = num(n2p) + n1t, n2tp = num(n1p) + n2t;
      double ca = R.J[n12t - 1] + R.J[n12p - 1] - R.J[n1tp - 1] - R.J[n2tp - 1];
      if (ns1t == ns2t) ca = ca - R.K[n12t - 1];
      if (ns1p == ns2p) ca = ca - R.K[n12p - 1];
      if (ns1t == ns2p) ca = ca + R.K[n1tp - 1];
      if (ns1p == ns2t) ca = ca + R.K[n2tp - 1];
      if (j == l) ca = 0.5 * ca;
      ab = ab + ca;
    }
  }
  return ab;
}

void read_vectors(Run& R, bool sym_variant);
void vectors_of_s(Run& R, bool sym_variant);
void s_space_ci(Run& R, bool sym_variant);
void zero_order(Run& R);

void read_inputs(Run& R, bool sym_variant) {
  const Options& o = R.o;
  if (o.yion) throw Error("yion (excitation to infinity) is not supported");
  if (o.isz != 0) throw Error("only isz = 0 is supported");
  if (o.ybrd && o.metat > 1) throw Error("ybrd (QDPT effective Hamiltonian) is not supported");
  if (o.ninact > 0) throw Error("ninact > 0 (restricted perturbation space) is not supported");
  if (o.lecdet < 2 || o.lecdet > 5) throw Error("lecdet 1 (determinants on cards) is not supported");
  if (o.ityper >= 0 && o.lecdet != 5 && R.device < 0)
    throw Error("a perturbation run with lecdet != 5 diagonalises S on the GPU: run it through cipsi_cip_main");
  if (o.metat < 1 || o.metat > 60) throw Error("trop d etats demandes en perturbation");
  auto recs = read_records(o.f40);
  if (recs.size() < 9) throw Error("unit 40 too short");
  {
    Record& h = recs[0];
    R.nsym = h.get<int32_t>();
    R.norb = h.get<int32_t>();
    R.noc = h.get<int32_t>();
    const int ntrans = h.get<int32_t>();
    R.itsym.resize(R.norb);
    for (auto& x : R.itsym) x = h.get<int32_t>();
    (void)h.get<int32_t>();
    R.ydp = h.get<uint8_t>() != 0;
    if (o.ydp >= 0) R.ydp = o.ydp != 0;  // ydp of &icinp is read after the header (deter.f:119,222)
    if (ntrans != 0) throw Error("degeneracy operations (ntrans > 0) are not supported");
  }
  R.its.resize((size_t)R.nsym * R.nsym);
  for (auto& x : R.its) x = recs[1].get<int32_t>();
  const size_t nter = (size_t)R.norb * (R.norb + 1) / 2;
  R.J.resize(nter);
  R.K.resize(nter);
  R.F.resize(nter);
  for (auto& x : R.J) x = recs[3].get<double>();
  for (auto& x : R.K) x = recs[4].get<double>();
  for (auto& x : R.F) x = recs[5].get<double>();
  for (auto& x : R.F)
    if (std::fabs(x) < 1.0e-10) x = 0.0;  // ijkf.f:34-37
  R.ij0.resize((size_t)R.norb * R.norb);
  for (auto& x : R.ij0) x = recs[6].get<int16_t>();
  const int ninte = recs[7].get<int32_t>();
  R.ntttt.resize(R.nsym);
  for (auto& x : R.ntttt) x = recs[7].get<int32_t>();
  R.eri.assign((size_t)ninte, 0.f);
  size_t pos = 0;
  const size_t nbuf = (size_t)ninte / 8192 + 1;
  if (recs.size() < 8 + nbuf) throw Error("unit 40: missing integral records");
  for (size_t b = 0; b < nbuf; ++b)
    for (int i = 0; i < 8192 && pos < (size_t)ninte; ++i, ++pos)
      R.eri[pos] = R.ydp ? (float)recs[8 + b].get<double>() : recs[8 + b].get<float>();
  if (o.ytocom) {  // deter.f:228-229: Fock-operator occupations from unit 21
    auto r21 = read_records(o.f21);
    if (r21.empty()) throw Error("unit 21: no occupation record");
    R.tocom21.resize(R.norb);
    for (auto& x : R.tocom21) x = r21[0].get<double>();
  }
  R.fdiag.assign(2 * R.norb, 0.0);
  for (int i = 1; i <= R.norb; ++i) R.fdiag[i - 1] = R.fdiag[i - 1 + R.norb] = R.F[(size_t)i * (i + 1) / 2 - 1];

  build_space(R, o.lecdet == 4 ? cas_space(R) : read_unit60(R, o.f60));
  // escf (rdener.f)
  bool found = false;
  for (auto& r : read_records(o.f33)) {
    if (r.b.size() >= 48 && std::memcmp(r.b.data(), "energie du determinant de reference     ", 40) == 0) {
      r.pos = 40;
      (void)r.get<int32_t>();
      R.escf = r.get<double>();
      found = true;
      break;
    }
  }
  if (!found) throw Error("energie du determinant de reference n'existe pas sur 33");
  if (o.ityper < 0) {
    // ic001 is not called (cip.f:71): c and e stay zero
    R.metat = o.metat;
    R.c.assign((size_t)R.ncf * R.metat, 0.0);
    R.e.assign(R.metat, 0.0);
  } else if (o.lecdet != 5) {
    s_space_ci(R, sym_variant);
  } else {
    read_vectors(R, sym_variant);
  }
  zero_order(R);
}

// degen (brdnee.f:299-365), called by ic001 once the vectors are read: a
// root m whose energy is within 1e-6 of the next root's, and not of the one
// after (a run of exactly two; the scan never pairs the last two roots, and
// longer runs are left alone), is rotated with root m+1 by the angle that
// gives the first spin-flip pair of unequal weights on root m equal weights
// (to 1e-4), if such a pair exists.
void rotate_degenerate_roots(Run& R) {
  const int ncf = R.ncf, metat = R.metat;
  const auto& e = R.e;
  int last = -1;  // 0-based index of the last root of the latest degenerate run
  for (int m = 0; m + 1 < metat; ++m) {
    if (m <= last) continue;
    int n = m + 1;
    while (n < metat && std::fabs(e[n] - e[m]) <= 1.0e-6) ++n;
    last = n == metat ? n - 2 : n - 1;  // a run reaching the last root ends one early
    if (last != m + 1) continue;        // no pair, or more than two degenerate roots
    double* c1v = R.c.data() + (size_t)m * ncf;
    double* c2v = c1v + ncf;
    bool rotated = false;
    for (int k = 0; k < ncf && !rotated; ++k) {
      if (R.S.ysaut[k] || R.S.nesp[k] == 0) continue;
      for (int ll = 1; ll <= R.S.nesp[k]; ++ll) {
        const double c11 = c1v[k], c12 = c1v[k + ll];
        if (std::fabs(std::fabs(c11) - std::fabs(c12)) < 1.0e-5) continue;
        const double c21 = c2v[k], c22 = c2v[k + ll], cc = c21 + c22;
        if (std::fabs(cc) < 1.0e-8) continue;
        const double phi = std::atan(-(c11 + c12) / cc), cs = std::cos(phi), si = std::sin(phi);
        const double a1 = std::fabs(c11 * cs + c21 * si), a2 = std::fabs(c12 * cs + c22 * si);
        if (std::fabs(a1 - a2) >= 1.0e-4) continue;
        for (int i = 0; i < ncf; ++i) {
          const double a = c1v[i] * cs + c2v[i] * si;
          c2v[i] = -c1v[i] * si + c2v[i] * cs;
          c1v[i] = a;
        }
        rotated = true;
        break;
      }
    }
  }
}

// ic001.f:44-76 (lecdet = 5): the vectors and energies of S from unit 59,
// in the order of unit 4's iord60 for cip; generators from them
void read_vectors(Run& R, bool sym_variant) {
  const Options& o = R.o;
  auto r4 = read_records(o.f04);
  if (r4.empty()) throw Error("unit 4 is empty");
  for (int i = 0; i < 4; ++i) (void)r4[0].get<int32_t>();
  const int mcf = r4[0].get<int32_t>();
  std::vector<int32_t> iord60;
  if (!sym_variant) {
    if (r4.size() < 2) throw Error("unit 4: missing iord60 record");
    iord60.resize(mcf);
    for (auto& x : iord60) x = r4[1].get<int32_t>();
  }
  auto r59 = read_records(o.f59);
  if (r59.empty()) throw Error("unit 59 is empty");
  const int ncf59 = r59[0].get<int32_t>();
  R.metat = r59[0].get<int32_t>();
  if (ncf59 != R.ncf) throw Error("files 59 and S incompatibles");
  if (R.metat < 1 || R.metat > CIPSI_MAX_ROOTS) throw Error("metat outside [1, 8]");
  R.c.resize((size_t)R.ncf * R.metat);
  for (auto& x : R.c) x = r59[0].get<double>();
  R.e.resize(R.metat);
  for (auto& x : R.e) x = r59[0].get<double>() - R.escf;
  if (mcf != R.ncf) throw Error("files 4 et 59 incompatibles");
  if (!sym_variant) {
    std::vector<double> tmp(R.ncf);
    for (int m = 0; m < R.metat; ++m) {
      for (int k = 0; k < R.ncf; ++k) tmp[iord60[k] - 1] = R.c[(size_t)m * R.ncf + k];
      for (int k = 0; k < R.ncf; ++k) R.c[(size_t)m * R.ncf + k] = tmp[k];
    }
  }
  vectors_of_s(R, sym_variant);
}

// after the vectors of S are known (ic001.f): degen, then the generators --
// every determinant for cipsym (cipsym/ic001.f:179), those with |c| >= coeff
// on some root for cip (cip/ic001.f:751)
void vectors_of_s(Run& R, bool sym_variant) {
  rotate_degenerate_roots(R);
  for (int k = 0; k < R.ncf; ++k) {
    if (sym_variant) {
      R.S.ygen[k] = 1;
    } else {
      for (int m = 0; m < R.metat; ++m)
        if (std::fabs(R.c[(size_t)m * R.ncf + k]) >= R.o.coeff) R.S.ygen[k] = 1;
    }
  }
}

// ic001.f:81-131 (lecdet != 5, ityper >= 0): H over S -- hdig on the
// diagonal, hntd within two excitations -- and its lowest metat eigenpairs.
// The pairs come from cipsi_hamiltonian_build on the run's GPU, the
// eigenpairs from cipsi_davidson (residuals converged to 1e-13 of H's
// largest diagonal element)
// instead of the reference's LAPACK call (diagonaliser.f90).  Each
// vector's first component of magnitude above 1e-8 of its largest is made
// positive (LAPACK's signs are its own; E2 and the selection use
// <I|H|Psi>^2).
void s_space_ci(Run& R, bool sym_variant) {
  const int n = R.ncf;
  R.metat = std::min(R.o.metat, n);
  if (R.metat > CIPSI_MAX_ROOTS) throw Error("the S diagonalisation takes at most 8 roots");
  cipsi_dims d{};
  d.norb = R.norb;
  d.noca = R.noc;
  d.nsym = R.nsym;
  d.isym = R.isym > 0 ? R.isym : 1;
  d.isz = 0;
  d.metat = 1;
  d.ncf = n;
  cipsi_ctx* ctx = nullptr;
  struct Guard {
    cipsi_ctx*& c;
    ~Guard() { if (c) cipsi_ctx_destroy(c); }
  } guard{ctx};
  auto chk = [&](int code, const char* what) {
    if (code) throw Error(std::string(what) + ": " + cipsi_last_error(ctx));
  };
  chk(cipsi_ctx_create(&ctx, &d, R.device), "cipsi_ctx_create");
  chk(cipsi_set_integrals(ctx, R.itsym.data(), R.its.data(), R.F.data(), R.J.data(), R.K.data(), R.ij0.data(),
                          R.ntttt.data(), R.eri.data(), (int64_t)R.eri.size()),
      "cipsi_set_integrals");
  chk(cipsi_set_space(ctx, R.S.ne.data(), R.S.nd.data(), R.S.trou.data(), R.S.part.data(), (int64_t)R.S.trou.size(),
                      R.S.ygen.data(), R.S.ysaut.data(), R.S.nesp.data(), R.S.yef1.data()),
      "cipsi_set_space");
  int64_t npairs = 0;
  chk(cipsi_hamiltonian_build(ctx, nullptr, -1, &npairs), "cipsi_hamiltonian_build");
  std::vector<int64_t> rowptr((size_t)n + 1);
  std::vector<int32_t> col((size_t)std::max<int64_t>(npairs, 1));
  std::vector<double> val((size_t)std::max<int64_t>(npairs, 1));
  chk(cipsi_hamiltonian_get(ctx, 0, n, rowptr.data(), col.data(), val.data()), "cipsi_hamiltonian_get");
  cipsi_ctx_destroy(ctx);
  ctx = nullptr;
  std::vector<int32_t> I, J;
  std::vector<double> V;
  I.reserve((size_t)npairs + n);
  J.reserve((size_t)npairs + n);
  V.reserve((size_t)npairs + n);
  for (int i = 0; i < n; ++i) {
    for (int64_t t = rowptr[i]; t < rowptr[i + 1]; ++t) {
      I.push_back(i + 1);
      J.push_back(col[t] + 1);
      V.push_back(val[t]);
    }
    I.push_back(i + 1);
    J.push_back(i + 1);
    V.push_back(0.5 * hdig_list(R, i));  // cipsi_davidson takes the diagonal halved
  }
  // residuals converged to 1e-13 of the largest diagonal element (about
  // what double precision resolves), so the vectors agree with a dense
  // solver's to ~1e-13 and E2 to ~1e-12 of itself
  double hmax = 1.0;
  for (int i = 0; i < n; ++i) hmax = std::max(hmax, std::fabs(hdig_list(R, i)));
  std::vector<double> ev(R.metat), vec((size_t)n * R.metat);
  char derr[512] = {0};
  int iters = 0;
  if (cipsi_davidson(n, (int64_t)V.size(), I.data(), J.data(), V.data(), R.metat, 1.0e-13 * hmax, 5000, R.device,
                     ev.data(), vec.data(), &iters, nullptr, derr, (int32_t)sizeof derr))
    throw Error(derr);
  R.e = ev;
  R.c = vec;
  for (int m = 0; m < R.metat; ++m) {
    double* x = R.c.data() + (size_t)m * n;
    double big = 0.0;
    for (int i = 0; i < n; ++i) big = std::max(big, std::fabs(x[i]));
    double sg = 1.0;
    for (int i = 0; i < n; ++i)
      if (std::fabs(x[i]) > 1e-8 * big) {
        sg = x[i] < 0.0 ? -1.0 : 1.0;
        break;
      }
    for (int i = 0; i < n; ++i) x[i] *= sg;
  }
  std::printf(" nombre de determinants   ncf=%9d\n valeurs propres\n", n);
  for (double x : R.e) std::printf(" %12.8f", x);
  std::printf("\n");
  vectors_of_s(R, sym_variant);
}

// faifoc.f and the zero-order quantities of cip.f:75-135
void zero_order(Run& R) {
  const Options& o = R.o;
  // faifoc.f with the occupations of cip.f:75-84
  std::vector<double> tocom(2 * R.norb, 0.0);
  for (int i = 0; i < R.noc; ++i) tocom[i] = 2.0;
  for (auto& e : o.tocom)
    if (e.first <= R.norb) tocom[e.first - 1] = e.second;
  for (size_t i = 0; i < R.tocom21.size(); ++i) tocom[i] = R.tocom21[i];
  for (int i = 0; i < R.norb; ++i) {
    if (tocom[i] > 1.0) {
      tocom[i + R.norb] = tocom[i] - 1.0;
      tocom[i] = 1.0;
    } else {
      tocom[i + R.norb] = 0.0;
    }
  }
  for (int i = 0; i < R.noc; ++i) {
    tocom[i] -= 1.0;
    tocom[i + R.norb] -= 1.0;
  }
  R.fmpb.assign(2 * R.norb, 0.0);
  auto num = [](int i) { return i * (i - 1) / 2; };
  for (int l = 1; l <= R.norb; ++l) {
    double t = R.fdiag[l - 1];
    int lj = num(l);
    for (int j = 1; j <= R.norb; ++j) {
      lj = lj + 1;
      if (j > l) lj = num(j) + l;
      t = t + (tocom[j - 1] + tocom[j - 1 + R.norb]) * R.J[lj - 1];
    }
    double tt = t;
    lj = num(l);
    for (int j = 1; j <= R.norb; ++j) {
      lj = lj + 1;
      if (j > l) lj = num(j) + l;
      t = t - tocom[j - 1] * R.K[lj - 1];
      tt = tt - tocom[j - 1 + R.norb] * R.K[lj - 1];
    }
    R.fmpb[l - 1] = t;
    R.fmpb[l - 1 + R.norb] = tt;
  }
  for (int i = 0; i < R.norb; ++i) {
    R.fmpb[i] = (R.fmpb[i] + R.fmpb[i + R.norb]) * 0.5;
    R.fmpb[i + R.norb] = R.fmpb[i];
  }
  // zero order (cip.f:99-135)
  R.emp.assign(R.metat, 0.0);
  R.eb.assign(R.metat, 0.0);
  R.teste.assign(R.metat, o.test);
  R.taum.assign(R.metat, 1.0);
  R.tocom = tocom;
  std::vector<double>& empdet = R.empdet;
  empdet.assign(R.ncf, 0.0);
  std::vector<double>& hdiag = R.hdiag;
  hdiag.assign(R.ncf, 0.0);
  for (int k = 0; k < R.ncf; ++k) {
    empdet[k] = hmp_list(R, k);
    hdiag[k] = hdig_list(R, k);
  }
  const bool yselm = o.iselec == 1;
  for (int m = 0; m < R.metat; ++m) {
    double t = 0.0;
    for (int i = 0; i < R.ncf; ++i) {
      const double ci = R.c[(size_t)m * R.ncf + i];
      if (!(t > std::fabs(ci))) t = std::fabs(ci);
      R.emp[m] = R.emp[m] + ci * ci * empdet[i];
      R.eb[m] = R.eb[m] + (ci * ci * hdiag[i]);
    }
    if (yselm) {
      R.teste[m] = t * o.test;
      if (o.ityper >= 0) R.taum[m] = 1.0 / t;
    }
  }
}

// ------------------------------------------------------------------ unit 4
// dimension of nblock / nstart in the reference's parameter file (pshf.prm
// ndetz): the zero-order record carries both arrays in full
constexpr int kUnit4Ndetz = 500000;

bool yocd_of(const Run& R, int so, int k) {
  for (int l = 0; l < R.S.ne[k]; ++l)
    if (R.S.trou[R.S.nd[k] + l] == so || R.S.part[R.S.nd[k] + l] == so) return true;
  return false;
}

// cip.f:136-150: the zero-order record that cip writes on unit 4 (rewinding
// it) before the perturbation
void write_unit4_zero_order(const Run& R) {
  std::FILE* f = std::fopen(R.o.f04.c_str(), "wb");
  if (!f) throw Error("cannot rewrite " + R.o.f04);
  const int ncf = R.ncf, mt = R.metat, n = R.norb, mn = 2 * R.norb;
  // the reference's list offsets (transf.f:26-29, 86-87): a determinant
  // without excitations (the reference) still takes one zero slot
  std::vector<int32_t> ndr(ncf), tr, pa;
  for (int k = 0; k < ncf; ++k) {
    ndr[k] = (int32_t)tr.size();
    if (R.S.ne[k] == 0) {
      tr.push_back(0);
      pa.push_back(0);
    }
    for (int l = 0; l < R.S.ne[k]; ++l) {
      tr.push_back(R.S.trou[R.S.nd[k] + l]);
      pa.push_back(R.S.part[R.S.nd[k] + l]);
    }
  }
  const int jj = ncf * mt, ii = ndr[ncf - 1] + R.S.ne[ncf - 1] + 1;
  const double e0 = R.o.ityper == 0 ? R.escf : 0.0;
  RecWriter w;
  for (int32_t v : {(int32_t)n, (int32_t)R.noc, (int32_t)(R.noc + n), (int32_t)mt, (int32_t)ncf, (int32_t)0})
    w.put<int32_t>(v);
  w.put<uint8_t>(0);  // yion
  w.put<int32_t>(ii);
  w.put<int32_t>(jj);
  for (int k = 0; k < ncf; ++k) {
    w.put<int32_t>(R.S.ne[k]);
    w.put<int32_t>(ndr[k]);
  }
  for (int j = 0; j < ii; ++j) {
    const bool in = j < (int)tr.size();
    w.put<int32_t>(in ? tr[j] : 0);
    w.put<int32_t>(in ? pa[j] : 0);
  }
  for (int j = 0; j < jj; ++j) w.put<double>(R.c[j]);
  for (int m = 0; m < mt; ++m) w.put<double>(R.e[m] + e0);
  for (int m = 0; m < mt; ++m) w.put<double>(R.emp[m]);
  for (int m = 0; m < mt; ++m) w.put<double>(R.eb[m]);
  for (int m = 0; m < mt; ++m) w.put<int32_t>(state_number(R.o, m));
  for (int k = 0; k < ncf; ++k) w.put<double>(R.empdet[k]);
  for (int i = 0; i < n; ++i) w.put<double>(R.fmpb[i]);
  for (int i = 0; i < n; ++i) w.put<double>(R.tocom[i]);
  for (int i = 0; i < 2 * kUnit4Ndetz; ++i) w.put<int32_t>(0);  // nblock, nstart (given.f): unused, lecdet = 5
  for (int i = 1; i <= mn; ++i) w.put<int32_t>(i <= n ? i : i - n);  // iorb
  for (int i = 1; i <= mn; ++i) w.put<int32_t>(i <= n ? 0 : 1);      // ispin
  for (int k = 0; k < ncf; ++k)
    for (int so = 1; so <= mn; ++so) w.put<uint8_t>(yocd_of(R, so, k) ? 1 : 0);
  w.flush(f);
  std::fclose(f);
}

// brdnee.f:38-135 for the spin flip alone (isz = 0, no spatial operation):
// the signed index of the flipped image of every determinant of S and the
// sign of each root under the flip
std::vector<int> root_flip_signs(const Run& R) {
  const int ncf = R.ncf, n = R.norb;
  auto flip = [&](int so) { return so <= n ? so + n : so - n; };
  std::vector<int> itk(ncf, 0);  // 1-based signed image, 0 = none
  for (int k = 0; k < ncf; ++k) {
    if (R.S.ysaut[k]) continue;
    const int nespk = R.S.nesp[k] + 1, nec = R.S.ne[k];
    if (nec == 0) {
      itk[k] = k + 1;
      continue;
    }
    for (int kg = 0; kg < nespk; ++kg) {
      const int kk = k + kg, ndk = R.S.nd[kk];
      int ntl[16], npl[16], ncr = 1, ii = kk + 1;
      for (int i = 0; i < nec; ++i) {
        ntl[i] = flip(R.S.trou[ndk + i]);
        npl[i] = flip(R.S.part[ndk + i]);
      }
      bool sort = true;
      if (R.S.yef1[k]) {
        bool found = false;
        for (int ig = 0; ig < nespk && !found; ++ig) {
          ii = k + ig + 1;
          bool all = true;
          for (int i = 0; i < nec && all; ++i)
            if (!yocd_of(R, ntl[i], ii - 1) || !yocd_of(R, npl[i], ii - 1)) all = false;
          found = all;
        }
        if (!found && nec == 1) sort = false;
      }
      if (sort)
        for (int i = 0; i < nec - 1; ++i)
          for (int j = i + 1; j < nec; ++j) {
            if (!(ntl[j] > ntl[i])) { std::swap(ntl[i], ntl[j]); ncr = -ncr; }
            if (!(npl[j] > npl[i])) { std::swap(npl[i], npl[j]); ncr = -ncr; }
          }
      itk[kk] = ncr < 0 ? -ii : ii;
    }
  }
  std::vector<int> itm(R.metat, 1);
  for (int m = 0; m < R.metat; ++m) {
    const double* cm = R.c.data() + (size_t)m * ncf;
    double x = 0.0;
    for (int k = 0; k < ncf; ++k) {
      if (itk[k] == 0) continue;
      const int ik = std::abs(itk[k]) - 1;
      double ckk = cm[k] * cm[ik];
      if (itk[k] < 0) ckk = -ckk;
      x = x + ckk;
    }
    itm[m] = x < 0.0 ? -1 : 1;
  }
  return itm;
}

// The two effective-Hamiltonian records appended to unit 4: the zero-order
// one (packed triangle hz, escf, ityper, the root signs) and the perturbed
// ones (hm, hv, hb: MP, EN eigenvalue, EN barycentric)
void write_unit4_heff(const Run& R, const std::vector<double>& hz, const std::vector<double>& hm,
                      const std::vector<double>& hv, const std::vector<double>& hb,
                      const std::vector<int>& itm) {
  std::FILE* f = std::fopen(R.o.f04.c_str(), "ab");
  if (!f) throw Error("cannot append to " + R.o.f04);
  const int mt = R.metat;
  RecWriter w;
  for (double x : hz) w.put<double>(x);
  w.put<double>(R.escf);
  w.put<int32_t>(R.o.ityper);
  w.put<int32_t>(1);  // ntrsy: the spin flip alone
  for (int m = 0; m < mt; ++m) w.put<int32_t>(itm[m]);
  w.flush(f);
  for (double x : hm) w.put<double>(x);
  for (double x : hv) w.put<double>(x);
  for (double x : hb) w.put<double>(x);
  w.flush(f);
  std::fclose(f);
}

// cip.f:300-306 and 403-414: zero-order and perturbed effective Hamiltonians
// (diagonal without QDPT) appended to unit 4 after the perturbation
void write_unit4_results(const Run& R, const double* e2mp, const double* e2vp, const double* e2b,
                         const std::vector<int>& itm) {
  const int mt = R.metat, nbr = mt * (mt + 1) / 2;
  std::vector<double> hz(nbr, 0.0), hm(nbr, 0.0), hv(nbr, 0.0), hb(nbr, 0.0);
  for (int m = 1; m <= mt; ++m) {
    const int mm = m * (m + 1) / 2 - 1;
    const double eabs = R.e[m - 1] + R.escf;
    hm[mm] = eabs + e2mp[m - 1];
    hv[mm] = eabs + e2vp[m - 1];
    hb[mm] = eabs + e2b[m - 1];
    hz[mm] = eabs - R.escf;
  }
  write_unit4_heff(R, hz, hm, hv, hb, itm);
}

// shell.f: the order of S by increasing diagonal energy that cip.f:200-206
// takes before writing S alone: Shell's diminishing-increment sort of -hdig
// into decreasing order, increments n/2, n/4, .. (log2 n passes, the count
// from single-precision logarithms as shell.f computes it).  Ties keep the
// positions this sequence of exchanges gives them, so the order is the
// reference's even among equal energies.  Returns 0-based indices of S.
std::vector<int> energy_order(const Run& R) {
  const int n = R.ncf;
  std::vector<double> a(R.hdiag.size());
  std::vector<int> ind(n);
  for (int k = 0; k < n; ++k) {
    a[k] = -R.hdiag[k];
    ind[k] = k;
  }
  const double aln2i = (double)(1.0f / 0.69314748f), tiny = (double)1.0e-5f;
  const int passes = (int)((double)std::log((float)n) * aln2i + tiny);
  int m = n;
  for (int pass = 0; pass < passes; ++pass) {
    m /= 2;
    for (int j = 0; j < n - m; ++j)
      for (int i = j; i >= 0 && a[i + m] > a[i]; i -= m) {
        std::swap(a[i], a[i + m]);
        std::swap(ind[i], ind[i + m]);
      }
  }
  return ind;
}

void write_pie_records(std::FILE* f, const std::vector<int32_t>& nec, const std::vector<int32_t>& h,
                       const std::vector<int32_t>& p, const std::vector<double>& v,
                       const std::vector<double>& evp, int metat, bool sym_variant, size_t hstride);

// unit 60 as pie.f writes it: the determinants of S in the given order, v = 1
long long write_space_unit60(std::FILE* f60, const Run& R, const std::vector<int>& order, bool sym_variant) {
  const size_t n = order.size();
  std::vector<int32_t> nec(n), h(n * 8, 0), p(n * 8, 0);
  std::vector<double> v(n, 1.0), ev(n * R.metat, 0.0);
  for (size_t q = 0; q < n; ++q) {
    const int k = order[q];
    nec[q] = R.S.ne[k];
    for (int l = 0; l < nec[q]; ++l) {
      h[q * 8 + l] = R.S.trou[R.S.nd[k] + l];
      p[q * 8 + l] = R.S.part[R.S.nd[k] + l];
    }
  }
  write_pie_records(f60, nec, h, p, v, ev, R.metat, sym_variant, 8);
  return (long long)n;
}

void write_pie_records(std::FILE* f, const std::vector<int32_t>& nec, const std::vector<int32_t>& h,
                       const std::vector<int32_t>& p, const std::vector<double>& v,
                       const std::vector<double>& evp, int metat, bool sym_variant, size_t hstride) {
  // cip/pie.f (cipsym/pie.f): records of at most lungo = 1000 determinants
  const size_t n = nec.size();
  for (size_t s = 0; s < n; s += 1000) {
    const size_t e = std::min(n, s + 1000);
    RecWriter w;
    int32_t m = 0;
    for (size_t i = s; i < e; ++i) m += 2 * nec[i];
    w.put<int32_t>(m);
    w.put<int32_t>((int32_t)(e - s));
    for (size_t i = s; i < e; ++i)
      for (int l = 0; l < nec[i]; ++l) {
        w.put<int32_t>(h[i * hstride + l]);
        w.put<int32_t>(p[i * hstride + l]);
      }
    for (size_t i = s; i < e; ++i) w.put<int32_t>(nec[i]);
    for (size_t i = s; i < e; ++i) w.put<double>(v[i]);
    if (sym_variant)
      for (size_t i = s; i < e; ++i)
        for (int q = 0; q < metat; ++q) w.put<double>(evp[i * metat + q]);
    w.flush(f);
  }
}

// Record consumer of cipsi_run_pt2_stream that writes the selected
// perturbers to unit 60 as pie.f does (cip/pie.f, cipsym/pie.f): records of
// lungo = 1000 determinants, each with its excitation list relative to the
// reference (holes and particles as 1-based spin orbitals, beta ones offset
// by norb), v = xam and, in cipsym, ENvp per root.  Pieces arrive in record
// order; a partial record waits for the next piece.
struct Unit60Writer {
  std::FILE* f;
  int norb, noca, metat;
  bool sym_variant;
  std::vector<int32_t> nec, h, p;
  std::vector<double> v, ev;
  int64_t written = 0;
  void add(int words, const uint64_t* bits, double xam, const double* evp) {
    const int W = words / 2;
    int nh = 0, np = 0;
    int32_t hh[8] = {0}, pp[8] = {0};
    for (int s = 0; s < 2; ++s)
      for (int w = 0; w < W; ++w) {
        const uint64_t word = bits[s * W + w];
        const int lo = w * 64;
        const int nref = std::min(std::max(noca - lo, 0), 64);
        const uint64_t ref = nref >= 64 ? ~0ull : ((1ull << nref) - 1ull);
        uint64_t hm = ref & ~word, pm = word & ~ref;
        while (hm) {
          const int b = __builtin_ctzll(hm);
          hm &= hm - 1;
          if (nh < 8) hh[nh] = lo + b + 1 + s * norb;
          ++nh;
        }
        while (pm) {
          const int b = __builtin_ctzll(pm);
          pm &= pm - 1;
          if (np < 8) pp[np] = lo + b + 1 + s * norb;
          ++np;
        }
      }
    if (nh > 8) throw Error("selected determinant with excitation degree > 8 (pie.f)");
    nec.push_back(nh);
    for (int l = 0; l < 8; ++l) {
      h.push_back(hh[l]);
      p.push_back(pp[l]);
    }
    v.push_back(xam);
    for (int m = 0; m < metat; ++m) ev.push_back(evp[m]);
    if (nec.size() == 1000) flush();
  }
  void flush() {
    if (nec.empty()) return;
    write_pie_records(f, nec, h, p, v, ev, metat, sym_variant, 8);
    written += (int64_t)nec.size();
    nec.clear(); h.clear(); p.clear(); v.clear(); ev.clear();
  }
};

int unit60_consumer(void* user, int64_t first, int64_t count, int32_t words, int32_t metat, const uint64_t* bits,
                    const int32_t* owner, const double* xam, const double* evp) {
  (void)first;
  (void)owner;
  Unit60Writer* w = static_cast<Unit60Writer*>(user);
  try {
    for (int64_t i = 0; i < count; ++i) w->add(words, bits + (size_t)i * words, xam[i], evp + (size_t)i * metat);
  } catch (const std::exception&) {
    return 1;
  }
  return 0;
}

std::string json_array(const double* x, int n) {
  std::ostringstream s;
  s.precision(17);
  s << "[";
  for (int i = 0; i < n; ++i) s << (i ? ", " : "") << x[i];
  s << "]";
  return s.str();
}

}  // namespace

struct cipsi_inputs {
  Run R;
  int sym_variant = 1;
};

namespace {

cipsi_opts opts_of(const Run& R, int sym_variant) {
  cipsi_opts op{};
  op.yen = R.o.ityper == 2;
  op.ysele = R.o.iselec == 3;
  op.ymoyen = R.o.ymoyen;
  op.ywdeg = R.o.ywdeg;
  op.sym_variant = sym_variant != 0;
  op.nclass = R.o.nclass;
  op.tau = R.o.tau;
  op.teseff = R.o.teseff;
  for (int i = 0; i < 10; ++i) op.aval[i] = R.o.aval[i];
  op.gen_mask = nullptr;
  op.run_pertu = 1;
  return op;
}

void seterr(char* errbuf, int32_t errlen, const std::string& m) {
  if (errbuf && errlen > 0) std::snprintf(errbuf, (size_t)errlen, "%s", m.c_str());
}

}  // namespace

namespace {
int inputs_read(cipsi_inputs** out, const char* workdir, const char* stdin_path, int32_t sym_variant, int device,
                char* errbuf, int32_t errlen);
}

extern "C" int cipsi_inputs_read(cipsi_inputs** out, const char* workdir, const char* stdin_path,
                                 int32_t sym_variant, char* errbuf, int32_t errlen) {
  return inputs_read(out, workdir, stdin_path, sym_variant, -1, errbuf, errlen);
}

namespace {
int inputs_read(cipsi_inputs** out, const char* workdir, const char* stdin_path, int32_t sym_variant, int device,
                char* errbuf, int32_t errlen) {
  if (!out) return CIPSI_ERR_ARG;
  *out = nullptr;
  try {
    const std::string dir = workdir ? workdir : ".";
    std::ifstream in(stdin_path ? std::string(stdin_path) : dir + "/cip.in");
    if (!in) throw Error("cannot read the namelist input");
    std::stringstream ss;
    ss << in.rdbuf();
    auto* h = new cipsi_inputs();
    h->sym_variant = sym_variant != 0;
    try {
      h->R.o = read_options(ss.str(), dir, sym_variant != 0);
      if (h->R.o.teseff < 0.0) h->R.o.teseff = 0.05 * h->R.o.tau;
      h->R.device = device;
      read_inputs(h->R, sym_variant != 0);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
    return CIPSI_OK;
  } catch (const std::exception& ex) {
    seterr(errbuf, errlen, ex.what());
    return CIPSI_ERR_ARG;
  }
}
}  // namespace

extern "C" void cipsi_inputs_free(cipsi_inputs* in) { delete in; }

extern "C" int cipsi_inputs_dims(const cipsi_inputs* in, cipsi_dims* dims, cipsi_opts* opts) {
  if (!in) return CIPSI_ERR_ARG;
  const Run& R = in->R;
  if (dims) *dims = cipsi_dims{R.norb, R.noc, R.nsym, R.isym ? R.isym : 1, 0, R.metat, R.ncf};
  if (opts) *opts = opts_of(R, in->sym_variant);
  return CIPSI_OK;
}

extern "C" int cipsi_inputs_array(const cipsi_inputs* in, const char* name, const void** data, int64_t* count,
                                  int32_t* type) {
  if (!in || !name || !data || !count || !type) return CIPSI_ERR_ARG;
  const Run& R = in->R;
  const std::string nm(name);
  auto put = [&](const auto& v, int t) {
    *data = v.data();
    *count = (int64_t)v.size();
    *type = t;
    return CIPSI_OK;
  };
  // type codes: 1 int32, 2 int16, 3 float32, 4 float64, 5 uint8
  if (nm == "itsym") return put(R.itsym, 1);
  if (nm == "its") return put(R.its, 1);
  if (nm == "ij0") return put(R.ij0, 2);
  if (nm == "ntttt") return put(R.ntttt, 1);
  if (nm == "F") return put(R.F, 4);
  if (nm == "J") return put(R.J, 4);
  if (nm == "K") return put(R.K, 4);
  if (nm == "eri") return put(R.eri, 3);
  if (nm == "c") return put(R.c, 4);
  if (nm == "e") return put(R.e, 4);
  if (nm == "eb") return put(R.eb, 4);
  if (nm == "emp") return put(R.emp, 4);
  if (nm == "teste") return put(R.teste, 4);
  if (nm == "taum") return put(R.taum, 4);
  if (nm == "fmpb") return put(R.fmpb, 4);
  if (nm == "ne") return put(R.S.ne, 1);
  if (nm == "nd") return put(R.S.nd, 1);
  if (nm == "trou") return put(R.S.trou, 1);
  if (nm == "part") return put(R.S.part, 1);
  if (nm == "ygen") return put(R.S.ygen, 5);
  if (nm == "ysaut") return put(R.S.ysaut, 5);
  if (nm == "nesp") return put(R.S.nesp, 1);
  if (nm == "yef1") return put(R.S.yef1, 5);
  if (nm == "escf") {
    *data = &R.escf;
    *count = 1;
    *type = 4;
    return CIPSI_OK;
  }
  return CIPSI_ERR_ARG;
}

extern "C" int cipsi_inputs_upload(const cipsi_inputs* in, cipsi_ctx* ctx) {
  if (!in || !ctx) return CIPSI_ERR_ARG;
  const Run& R = in->R;
  int rc = cipsi_set_integrals(ctx, R.itsym.data(), R.its.data(), R.F.data(), R.J.data(), R.K.data(),
                               R.ij0.data(), R.ntttt.data(), R.eri.data(), (int64_t)R.eri.size());
  if (rc) return rc;
  rc = cipsi_set_space(ctx, R.S.ne.data(), R.S.nd.data(), R.S.trou.data(), R.S.part.data(),
                       (int64_t)R.S.trou.size(), R.S.ygen.data(), R.S.ysaut.data(), R.S.nesp.data(),
                       R.S.yef1.data());
  if (rc) return rc;
  return cipsi_set_roots(ctx, R.c.data(), R.e.data(), R.eb.data(), R.emp.data(), R.teste.data(),
                         R.taum.data(), R.fmpb.data());
}

extern "C" int cipsi_cip_main(const char* workdir, const char* stdin_path, int32_t sym_variant,
                              const char* json_path, const uint8_t* gen_mask, int32_t device,
                              char* errbuf, int32_t errlen) {
  cipsi_ctx* ctx = nullptr;
  cipsi_inputs* in = nullptr;
  try {
    int rc = inputs_read(&in, workdir, stdin_path, sym_variant, device, errbuf, errlen);
    if (rc) return rc;
    const Run& R = in->R;
    const auto t0 = std::chrono::steady_clock::now();
    write_unit4_zero_order(R);  // cip.f:144, during the set-up
    if (R.o.ityper < 0) {
      // cip.f:200-236: S by increasing diagonal energy, the (empty) effective
      // Hamiltonians on unit 4, S on unit 60 when ymoyen, and stop: no
      // perturbation, no device work
      const int mt = R.metat, nbr = mt * (mt + 1) / 2;
      const std::vector<double> zero(nbr, 0.0);
      write_unit4_heff(R, zero, zero, zero, zero, root_flip_signs(R));
      long long ntot = 0;
      if (R.o.ymoyen) {
        std::FILE* f60 = std::fopen(R.o.f60.c_str(), "wb");
        if (!f60) throw Error("cannot rewrite " + R.o.f60);
        ntot = write_space_unit60(f60, R, energy_order(R), sym_variant != 0);
        std::fclose(f60);
      }
      if (json_path) {
        std::ofstream j(json_path);
        j << "{\n  \"ncf\": " << R.ncf << ", \"metat\": " << mt << ", \"norb\": " << R.norb
          << ", \"noca\": " << R.noc << ", \"ntot60\": " << ntot << "\n}\n";
      }
      cipsi_inputs_free(in);
      return 0;
    }
    cipsi_dims d{};
    cipsi_opts op{};
    cipsi_inputs_dims(in, &d, &op);
    op.gen_mask = gen_mask;
    auto chk = [&](int code, const char* what) {
      if (code) throw Error(std::string(what) + ": " + cipsi_last_error(ctx));
    };
    const std::vector<int> itm = root_flip_signs(R);
    cipsi_result res{};
    // unit 60 when ymoyen: S (v = 1) then the selected perturbers, streamed
    // from the GPU chunk by chunk and written while the next chunk computes;
    // without ymoyen the reference writes nothing to it (cip.f:222,
    // pert1.f:264)
    long long ntot = 0;
    std::FILE* f60 = nullptr;
    if (R.o.ymoyen) {
      f60 = std::fopen(R.o.f60.c_str(), "wb");
      if (!f60) throw Error("cannot rewrite " + R.o.f60);
      std::vector<int> identity(R.ncf);
      for (int k = 0; k < R.ncf; ++k) identity[k] = k;
      ntot += write_space_unit60(f60, R, identity, sym_variant != 0);
    }
    struct CloseFile {
      std::FILE*& f;
      ~CloseFile() { if (f) std::fclose(f); }
    } close60{f60};
    if (R.o.ityper != 0) {  // ityper = 0: no perturbation (deter.f:231), no device work
      chk(cipsi_ctx_create(&ctx, &d, device), "cipsi_ctx_create");
      chk(cipsi_inputs_upload(in, ctx), "cipsi_inputs_upload");
      if (f60) {
        Unit60Writer w{f60, R.norb, R.noc, R.metat, sym_variant != 0, {}, {}, {}, {}, {}, 0};
        chk(cipsi_run_pt2_stream(ctx, &op, 0, unit60_consumer, &w, &res), "cipsi_run_pt2_stream");
        w.flush();
        ntot += w.written;
      } else {
        chk(cipsi_run_pt2(ctx, &op, &res), "cipsi_run_pt2");
      }
    }
    if (f60) {
      std::fclose(f60);
      f60 = nullptr;
    }
    const auto t1 = std::chrono::steady_clock::now();
    write_unit4_results(R, res.e2mp, res.e2vp, res.e2b, itm);
    // listing lines the Autocip driver reads (cipsym/cip.f:253-254, cip.f:243-247)
    std::printf("0 ont ete generes:    %10lld  etats efficaces\n", (long long)res.ietat);
    std::printf(" la contribution du plus grand determinant non ecrit est %8.6f\n", res.dpivot);
    if (sym_variant) {
      std::printf("nombre de determinants sur la file 60\n");
      std::printf("%12lld%12d\n", ntot, R.metat);
    }
    // unit 33 (stkener.f: char*40 then the values, no count), and the
    // listing stkener prints for each record: the name, then a line with the
    // values alone -- the Autocip driver finds ' energies CIPSI envp' and
    // reads metat values list-directed from the next line
    // (Autocip_13/calcul.f90:373-378)
    std::FILE* f33 = std::fopen(R.o.f33.c_str(), "ab");
    if (!f33) throw Error("cannot append to " + R.o.f33);
    const char* names[4] = {"energies CIPSI var ", "energies CIPSI mpb ", "energies CIPSI envp", "energies CIPSI enb "};
    std::vector<double> etot(R.metat);
    for (int m = 0; m < R.metat; ++m) etot[m] = R.e[m] + R.escf;
    const double* vals[4] = {etot.data(), res.e2mp, res.e2vp, res.e2b};
    for (int q = 0; q < 4; ++q) {
      std::string typ = std::string(names[q]) + R.o.title;
      typ.resize(40, ' ');
      RecWriter w;
      w.put_bytes(typ.data(), 40);
      for (int m = 0; m < R.metat; ++m) w.put<double>(vals[q][m]);
      w.flush(f33);
      std::printf(" *************************************\n");
      std::printf(" %s stockee sur la file 33\n", typ.c_str());
      for (int m = 0; m < R.metat; ++m) std::printf(" %24.16E", vals[q][m]);
      std::printf("\n *************************************\n");
    }
    std::fclose(f33);
    std::fflush(stdout);
    if (json_path) {
      std::ofstream j(json_path);
      j.precision(17);
      const int mt = R.metat;
      j << "{\n  \"ncf\": " << R.ncf << ", \"metat\": " << mt << ", \"norb\": " << R.norb
        << ", \"noca\": " << R.noc << ",\n";
      j << "  \"ietat\": " << res.ietat << ", \"n_processed\": " << res.n_processed
        << ", \"ntot60\": " << ntot << ",\n";
      j << "  \"dpivot\": " << res.dpivot << ",\n";
      j << "  \"e2mp\": " << json_array(res.e2mp, mt) << ",\n";
      j << "  \"e2vp\": " << json_array(res.e2vp, mt) << ",\n";
      j << "  \"e2b\": " << json_array(res.e2b, mt) << ",\n";
      j << "  \"psimp\": " << json_array(res.psimp, mt) << ",\n";
      j << "  \"psivp\": " << json_array(res.psivp, mt) << ",\n";
      j << "  \"e\": " << json_array(R.e.data(), mt) << ",\n";
      j << "  \"emp\": " << json_array(R.emp.data(), mt) << ",\n";
      j << "  \"eb\": " << json_array(R.eb.data(), mt) << ",\n";
      j << "  \"nom\": [";
      for (int i = 0; i < R.o.nclass; ++i) j << (i ? ", " : "") << res.nom[i];
      j << "],\n  \"nam\": [";
      for (int m = 0; m < mt; ++m) {
        j << (m ? ", " : "") << "[";
        for (int i = 0; i < R.o.nclass; ++i) j << (i ? ", " : "") << res.nam[i * CIPSI_MAX_ROOTS + m];
        j << "]";
      }
      j << "],\n  \"tabmp\": [";
      for (int m = 0; m < mt; ++m) {
        j << (m ? ", " : "") << "[";
        for (int i = 0; i < R.o.nclass; ++i) j << (i ? ", " : "") << res.tabmp[i * CIPSI_MAX_ROOTS + m];
        j << "]";
      }
      j << "],\n  \"tabvp\": [";
      for (int m = 0; m < mt; ++m) {
        j << (m ? ", " : "") << "[";
        for (int i = 0; i < R.o.nclass; ++i) j << (i ? ", " : "") << res.tabvp[i * CIPSI_MAX_ROOTS + m];
        j << "]";
      }
      j << "],\n  \"n_candidates\": " << res.n_candidates << ", \"n_compares\": " << res.n_compares
        << ", \"n_pairs_1\": " << res.n_pairs_1 << ", \"n_pairs_2\": " << res.n_pairs_2
        << ", \"alg_bytes\": " << res.alg_bytes << ",\n  \"kernel_ms\": " << res.kernel_ms
        << ", \"wall_s\": " << std::chrono::duration<double>(t1 - t0).count() << "\n}\n";
    }
    cipsi_ctx_destroy(ctx);
    cipsi_inputs_free(in);
    return 0;
  } catch (const std::exception& ex) {
    seterr(errbuf, errlen, ex.what());
    if (ctx) cipsi_ctx_destroy(ctx);
    if (in) cipsi_inputs_free(in);
    return CIPSI_ERR_ARG;
  }
}
