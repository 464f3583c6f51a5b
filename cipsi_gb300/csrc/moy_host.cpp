// moy_host.cpp -- host side of the GPU drop-in for moy.exe: the Hamiltonian
// over S + the selected perturbers that cip wrote to unit 60, for the
// Davidson diagonalisation that follows (bd).
//
// Reads what the reference reads (namelists &moyfil and &moyen on standard
// input; the first record of unit 4, unit 40 ijkl, unit 60 det), builds the
// determinant list as moy/deter.f does, and writes what the reference writes:
// unit 64 (the list with its spin-orbital tables) and unit 61 (the lists one
// determinant at a time), unit 1 (H by rows in 8192-element records),
// unit 63 (MP diagonal energies, ystkmp), and, as moy/morue.f, the
// second-order energies of the determinants beyond S to unit 33 and to a
// fourth unit-4 record.  The pair scan and the off-diagonal elements -- the
// O(n^2) part -- run on the GPU (cipsi_hamiltonian_build, hbuild.cu); the
// diagonal, the file formats and morue's sums stay here.
//
// Followed sources: moy/moy.f (main flow 28-233), moy/openf.f, moy/deter.f
// (ntrans = 0: lines 28-70, 96-191 and the partner loop 200-270),
// moy/lec60.f, moy/transf.f, moy/pie.f, moy/ijkf.f, moy/reijkl.f,
// moy/hdig.f, moy/hmp.f, moy/morue.f, moy/stkener.f.

#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cipsi_gb300.h"
#include "host_io.h"

namespace {

using namespace cipsi_host;

constexpr int kLsize = 8192;      // moy/pshf.prm lsize: elements per unit-1 record
constexpr int kNdimh = 10000000;  // moy/pshf.prm ndimh: determinants at most

struct MoyRun {
  // &moyfil unit files
  std::string f01, f04, f33, f40, f60, f61, f63, f64;
  // &moyen
  double tau = 0.0;
  bool yecr = false, ystkmp = false, yrcmp = false, y_secd = false;
  std::string title = "                    ";
  // unit 4, first record
  int norb = 0, noca = 0, nocb = 0, metat = 1, ndims = 0, isz = 0;
  std::vector<double> c4, e4, ebmp, eben, fmpb;  // fmpb by spin orbital (0-based)
  // unit 40
  int nsym = 1;
  bool ydp = false;
  std::vector<int32_t> itsym, its;  // its column-major nsym x nsym
  std::vector<double> F, J, K, fdiag;
  std::vector<int16_t> ij0;
  std::vector<int32_t> ntttt;
  std::vector<float> eri;
  // the list (moy/pie.f: nd(k) = sum of ne(l < k), 0-based offsets)
  int isym = 0;
  std::vector<int32_t> ne, nd, trou, part;
  std::set<std::vector<int>> keys;
};

// moy/transf.f + pie.f: sort the holes and the particles, check the spin
// orbitals, refuse a determinant of another symmetry (the run goes on),
// drop a repeat, else append.  Returns true when appended.
bool transf(MoyRun& M, int nec, int* nt, int* np) {
  const int norb = M.norb, mnorb = 2 * norb, noca = M.noca, nocb = M.nocb;
  auto append = [&]() {
    std::vector<int> key(nt, nt + nec);
    key.insert(key.end(), np, np + nec);
    if (!M.keys.insert(std::move(key)).second) return false;
    M.ne.push_back(nec);
    M.nd.push_back((int)M.trou.size());
    for (int j = 0; j < nec; ++j) {
      M.trou.push_back(nt[j]);
      M.part.push_back(np[j]);
    }
    return true;
  };
  if (nec == 0) {
    M.isym = 1;
    if (M.isz != 0) return false;
    return append();
  }
  std::sort(nt, nt + nec);
  std::sort(np, np + nec);
  auto bad = [&]() { throw Error("1 spin orbitale est hors de l espace de base"); };
  if (nt[0] < 1 || np[nec - 1] > mnorb || nt[nec - 1] > nocb || np[nec - 1] <= noca) bad();
  int is = 1, ls = 0;
  for (int i = 0; i < nec; ++i) {
    if (!(nt[i] <= noca) && nt[i] < norb + 1) bad();
    if (!(np[i] > nocb)) {
      if (np[i] > norb) bad();
      if (np[i] <= noca) bad();
    }
    const int st = M.itsym[(nt[i] - 1) % norb], sp = M.itsym[(np[i] - 1) % norb];
    is = M.its[(size_t)(st - 1) * M.nsym + (is - 1)];
    is = M.its[(size_t)(sp - 1) * M.nsym + (is - 1)];
    ls += (np[i] > norb) - (nt[i] > norb);
  }
  if (M.isym == 0) M.isym = is;
  if (is != M.isym) {  // transf.f:90-95
    std::printf(" determinant de mauvaise symetrie\n");
    return false;
  }
  if (ls != M.isz) throw Error("mauvais spin");
  return append();
}

// spin flip of a spin orbital (moy/deter.f:160-170 with igela = 1,
// igelb = norb + 1): 0 when the partner lies outside the space
int flip(const MoyRun& M, int so) {
  const int norb = M.norb, i = so <= norb ? so : so - norb, k = i + norb;
  if ((k < M.nocb && i > M.noca) || (k > M.nocb && i < M.noca)) return 0;
  return so <= norb ? k : i;
}

// moy/lec60.f then the list loop of moy/deter.f: the reference determinant
// first (if present), then by excitation degree 1..6, each appended
// determinant followed by its spin-flip partner
void build_list(MoyRun& M) {
  auto recs = read_records(M.f60);
  bool hf = false;
  std::vector<std::vector<std::vector<int>>> byrank(7);
  for (auto& r : recs) {
    const int mw = r.get<int32_t>(), nw = r.get<int32_t>();
    if (mw < 0 || nw < 0) throw Error("unit 60: bad record");
    std::vector<int32_t> idot(mw), necst(nw);
    std::vector<double> vs(nw);
    for (auto& x : idot) x = r.get<int32_t>();
    for (auto& x : necst) x = r.get<int32_t>();
    for (auto& x : vs) x = r.get<double>();
    int myy = 0;
    for (int l = 0; l < nw; ++l) {
      const int nec = necst[l];
      if (nec > 6 || nec < 0)
        throw Error("erreur degre d excitation " + std::to_string(nec) + " depasse les possibilites du programme");
      if (myy + 2 * nec > mw) throw Error("unit 60: record shorter than its excitation degrees");
      if (vs[l] < M.tau) {
        myy += 2 * nec;
        continue;
      }
      if (nec == 0) {
        if (M.isz != 0) continue;
        if (hf) std::printf(" fondamental deja present\n");
        hf = true;
        continue;
      }
      std::vector<int> itab(2 * nec);
      for (int s = 0; s < nec; ++s) {
        itab[s] = idot[myy++];
        itab[s + nec] = idot[myy++];
      }
      byrank[nec].push_back(std::move(itab));
    }
  }
  if (hf) transf(M, 0, nullptr, nullptr);
  for (int nec = 1; nec <= 6; ++nec)
    for (auto& itab : byrank[nec]) {
      int nt[8], np[8];
      for (int l = 0; l < nec; ++l) {
        nt[l] = itab[l];
        np[l] = itab[l + nec];
      }
      if (!transf(M, nec, nt, np)) continue;
      if (M.isz != 0) continue;
      bool ok = true;
      for (int l = 0; l < nec && ok; ++l) {
        nt[l] = flip(M, nt[l]);
        np[l] = flip(M, np[l]);
        ok = nt[l] != 0 && np[l] != 0;
      }
      if (ok) transf(M, nec, nt, np);
    }
}

// moy/hdig.f and moy/hmp.f for determinant k of the list (energies relative
// to the reference determinant)
double hdig(const MoyRun& M, int k) {
  const int n = M.norb;
  auto num = [](int i) { return i * (i - 1) / 2; };
  double ab = 0.0;
  const int l1 = M.nd[k], nei = M.ne[k];
  for (int l = 0; l < nei; ++l) {
    int n1p = M.part[l1 + l], n1t = M.trou[l1 + l];
    ab = ab + M.fdiag[n1p - 1] - M.fdiag[n1t - 1];
    const int ns1t = n1t > n, ns1p = n1p > n;
    n1t = (n1t - 1) % n + 1;
    n1p = (n1p - 1) % n + 1;
    for (int j = 0; j <= l; ++j) {
      int n2t = M.trou[l1 + j], n2p = M.part[l1 + j];
      const int ns2t = n2t > n, ns2p = n2p > n;
      n2t = (n2t - 1) % n + 1;
      n2p = (n2p - 1) % n + 1;
      const int n12t = n2t > n1t ? num(n2t) + n1t : num(n1t) + n2t;
      const int n12p = n2p > n1p ? num(n2p) + n1p : num(n1p) + n2p;
      const int n1tp = num(n2p) + n1t, n2tp = num(n1p) + n2t;
      double ca = M.J[n12t - 1] + M.J[n12p - 1] - M.J[n1tp - 1] - M.J[n2tp - 1];
      if (ns1t == ns2t) ca = ca - M.K[n12t - 1];
      if (ns1p == ns2p) ca = ca - M.K[n12p - 1];
      if (ns1t == ns2p) ca = ca + M.K[n1tp - 1];
      if (ns1p == ns2t) ca = ca + M.K[n2tp - 1];
      if (j == l) ca = 0.5 * ca;
      ab = ab + ca;
    }
  }
  return ab;
}
double hmp(const MoyRun& M, int k) {
  double ac = 0.0;
  for (int l = 0; l < M.ne[k]; ++l) ac = ac + M.fmpb[M.part[M.nd[k] + l] - 1] - M.fmpb[M.trou[M.nd[k] + l] - 1];
  return ac;
}

void read_unit4(MoyRun& M) {
  auto recs = read_records(M.f04);
  if (recs.empty()) throw Error("fin de fichier sur 4");
  Record& r = recs[0];
  M.norb = r.get<int32_t>();
  M.noca = r.get<int32_t>();
  M.nocb = r.get<int32_t>();
  M.metat = r.get<int32_t>();
  M.ndims = r.get<int32_t>();
  M.isz = r.get<int32_t>();
  const bool yion = r.get<uint8_t>() != 0;
  const int ii = r.get<int32_t>(), jj = r.get<int32_t>();
  if (M.norb < 2 || M.norb > 128 || M.metat < 1 || M.metat > 60 || M.ndims < 0 || ii < 0 || jj < 0)
    throw Error("erreur fichier sur 4");
  if (yion) throw Error("yion is not supported");
  if (M.isz != 0) throw Error("only isz = 0 is supported");
  for (int i = 0; i < 2 * M.ndims + 2 * ii; ++i) (void)r.get<int32_t>();
  M.c4.resize(jj);
  for (auto& x : M.c4) x = r.get<double>();  // morue.f:29
  M.e4.resize(M.metat);
  M.ebmp.resize(M.metat);
  M.eben.resize(M.metat);
  for (auto& x : M.e4) x = r.get<double>();
  for (auto& x : M.ebmp) x = r.get<double>();
  for (auto& x : M.eben) x = r.get<double>();
  for (int m = 0; m < M.metat; ++m) (void)r.get<int32_t>();
  for (int i = 0; i < M.ndims; ++i) (void)r.get<double>();
  M.fmpb.assign(2 * M.norb, 0.0);
  for (int i = 0; i < M.norb; ++i) M.fmpb[i] = M.fmpb[i + M.norb] = r.get<double>();
}

void read_unit40(MoyRun& M) {
  auto recs = read_records(M.f40);
  if (recs.size() < 8) throw Error("unit 40: too few records");
  Record& h = recs[0];
  M.nsym = h.get<int32_t>();
  const int norb = h.get<int32_t>();
  if (norb != M.norb) throw Error("units 40 and 4 disagree on norb");
  (void)h.get<int32_t>();  // noc
  const int ntrans = h.get<int32_t>();
  if (M.nsym < 1 || M.nsym > 8) throw Error("nsym must be in [1, 8]");
  M.itsym.resize(norb);
  for (auto& x : M.itsym) x = h.get<int32_t>();
  (void)h.get<int32_t>();  // noa
  M.ydp = h.get<uint8_t>() != 0;
  if (ntrans != 0) throw Error("spatial degeneracy operations (ntrans > 0) are not supported");
  M.its.resize((size_t)M.nsym * M.nsym);
  for (auto& x : M.its) x = recs[1].get<int32_t>();
  // moy/ijkf.f: one record skipped (h), then J, K and F as they stand
  const size_t nter = (size_t)norb * (norb + 1) / 2;
  M.J.resize(nter);
  M.K.resize(nter);
  M.F.resize(nter);
  for (auto& x : M.J) x = recs[3].get<double>();
  for (auto& x : M.K) x = recs[4].get<double>();
  for (auto& x : M.F) x = recs[5].get<double>();
  M.fdiag.assign(2 * norb, 0.0);
  for (int i = 1; i <= norb; ++i) M.fdiag[i - 1] = M.fdiag[i - 1 + norb] = M.F[(size_t)i * (i + 1) / 2 - 1];
  // moy/reijkl.f
  M.ij0.resize((size_t)norb * norb);
  for (auto& x : M.ij0) x = recs[6].get<int16_t>();
  const int ninte = recs[7].get<int32_t>();
  M.ntttt.resize(M.nsym);
  for (auto& x : M.ntttt) x = recs[7].get<int32_t>();
  if (ninte < 1) throw Error("unit 40: no integrals");
  const int nbuf = ninte / kLsize + 1;
  if ((int)recs.size() < 8 + nbuf) throw Error("unit 40: missing integral buffers");
  M.eri.assign((size_t)nbuf * kLsize, 0.f);
  size_t pos = 0;
  for (int b = 0; b < nbuf; ++b)
    for (int i = 0; i < kLsize; ++i, ++pos)
      M.eri[pos] = M.ydp ? (float)recs[8 + b].get<double>() : recs[8 + b].get<float>();
  M.eri.resize((size_t)ninte);
}

// moy/morue.f:62-105 applied to the unit-1 elements in file order: the
// elements (k, i <= ndims) of a row k > ndims add c(i, m) h into cunt(m);
// the row's diagonal element closes it into the effective-Hamiltonian sums
struct Morue {
  const MoyRun& M;
  const std::vector<double>& stefen;
  const std::vector<double>& stefmp;
  std::vector<double> cunt, hefmp, hefen, hefenb;
  Morue(const MoyRun& m, const std::vector<double>& en, const std::vector<double>& mp)
      : M(m), stefen(en), stefmp(mp), cunt(m.metat, 0.0) {
    const int mmm = m.metat * (m.metat + 1) / 2;
    hefmp.assign(mmm, 0.0);
    hefen.assign(mmm, 0.0);
    hefenb.assign(mmm, 0.0);
  }
  void entry(int k, int i, double hij) {  // 1-based, as stored on unit 1
    const int ndims = M.ndims, mt = M.metat;
    if (k == 1) return;
    if (k == i && k > ndims) {
      const double stenk = stefen[k - 1], stmpk = stefmp[k - 1];
      const double enk2 = stenk + stenk, empk2 = stmpk + stmpk;
      int ii = 0;
      for (int m = 0; m < mt; ++m)
        for (int n = 0; n <= m; ++n, ++ii) {
          const double denb = M.eben[m] + M.eben[n] - enk2;
          const double dmp = M.ebmp[m] + M.ebmp[n] - empk2;
          const double den = M.e4[m] + M.e4[n] - enk2;
          double hmn = cunt[m] * cunt[n];
          hmn = hmn + hmn;
          hefmp[ii] = hefmp[ii] + hmn / dmp;
          hefen[ii] = hefen[ii] + hmn / den;
          hefenb[ii] = hefenb[ii] + hmn / denb;
        }
      std::fill(cunt.begin(), cunt.end(), 0.0);
      return;
    }
    if (k <= ndims || i > ndims) return;
    for (int m = 0; m < mt; ++m) cunt[m] = cunt[m] + M.c4[(size_t)m * ndims + (i - 1)] * hij;
  }
};

// unit 1 (moy.f:150-184): (itab, jtab, vbuf) records of kLsize elements;
// the last record has itab(lsize) = -1 and jtab(lsize) = its element count,
// with the rest of its arrays left from the record before
struct Unit1Writer {
  std::FILE* f = nullptr;
  std::vector<int32_t> itab = std::vector<int32_t>(kLsize, 0), jtab = std::vector<int32_t>(kLsize, 0);
  std::vector<double> vbuf = std::vector<double>(kLsize, 0.0);
  int nbuf = 0;
  long long records = 0;
  Morue* morue = nullptr;
  void write() {
    const int32_t n = kLsize * 16;
    std::fwrite(&n, 4, 1, f);
    std::fwrite(itab.data(), 4, kLsize, f);
    std::fwrite(jtab.data(), 4, kLsize, f);
    std::fwrite(vbuf.data(), 8, kLsize, f);
    std::fwrite(&n, 4, 1, f);
    ++records;
  }
  void add(int i, int j, double h) {
    itab[nbuf] = i;
    jtab[nbuf] = j;
    vbuf[nbuf] = h;
    ++nbuf;
    if (morue) morue->entry(i, j, h);
    if (nbuf < kLsize) return;
    write();
    nbuf = 0;
  }
  void finish() {
    itab[kLsize - 1] = -1;
    jtab[kLsize - 1] = nbuf;
    write();
    // morue.f:66-70 reads a last record holding no element as if its first
    // element (left from the record before) were one more element
    if (morue && nbuf == 0 && records > 1) morue->entry(itab[0], jtab[0], vbuf[0]);
  }
};

void stkener(const MoyRun& M, const std::string& name, const std::vector<double>& x) {
  std::FILE* f33 = std::fopen(M.f33.c_str(), "ab");
  if (!f33) throw Error("cannot append to " + M.f33);
  std::string typ = name;
  typ.resize(40, ' ');
  RecWriter w;
  w.put_bytes(typ.data(), 40);
  for (double v : x) w.put<double>(v);
  w.flush(f33);
  std::fclose(f33);
  std::printf(" *************************************\n");
  std::printf(" %s stockee sur la file 33", typ.c_str());
  for (double v : x) std::printf(" %24.16E", v);
  std::printf("\n *************************************\n");
}

void seterr(char* errbuf, int32_t errlen, const std::string& m) {
  if (errbuf && errlen > 0) std::snprintf(errbuf, (size_t)errlen, "%s", m.c_str());
}

std::string json_array(const std::vector<double>& x) {
  std::ostringstream s;
  s.precision(17);
  s << "[";
  for (size_t i = 0; i < x.size(); ++i) s << (i ? ", " : "") << x[i];
  s << "]";
  return s.str();
}

}  // namespace

extern "C" int cipsi_moy_main(const char* workdir, const char* stdin_path, const char* json_path, int32_t device,
                              char* errbuf, int32_t errlen) {
  cipsi_ctx* ctx = nullptr;
  try {
    const auto t0 = std::chrono::steady_clock::now();
    const std::string dir = workdir ? workdir : ".";
    std::string text;
    {
      std::ifstream in(stdin_path ? stdin_path : "/dev/stdin");
      std::stringstream ss;
      ss << in.rdbuf();
      text = ss.str();
    }
    MoyRun M;
    // openf.f
    const std::set<std::string> moyfil = {"prefix", "det", "ijkl", "f04", "det1", "ijkl1", "f041",
                                          "det_cl", "det_spin", "mat", "enmp", "csf", "det_cl1",
                                          "mat1", "enmp1", "ener", "ener1", "csf1", "det_spin1"};
    Namelist cf = parse_namelist(text, "moyfil", moyfil);
    M.f01 = unit_file(cf, "mat", "mat1", "mat", dir);
    M.f04 = unit_file(cf, "f04", "f041", "f04", dir);
    M.f33 = unit_file(cf, "ener", "ener1", "ener", dir);
    M.f40 = unit_file(cf, "ijkl", "ijkl1", "ijkl", dir);
    M.f60 = unit_file(cf, "det", "det1", "det", dir);
    M.f61 = unit_file(cf, "det_cl", "det_cl1", "det_cl", dir);
    M.f63 = unit_file(cf, "enmp", "enmp1", "enmp", dir);
    M.f64 = unit_file(cf, "det_spin", "det_spin1", "det_spin", dir);
    read_unit4(M);
    // &moyen (moy.f:29-48)
    const std::set<std::string> moyen = {"yprt", "tau", "yecr", "ystkmp", "ymat", "iord", "title",
                                         "yrcmp", "y_secd", "yspipro", "ysymat"};
    Namelist nm = parse_namelist(text, "moyen", moyen);
    if (!nm.found) throw Error("erreur dans la namelist moyen");
    if (auto v = nm.scalar("tau")) M.tau = to_real(*v);
    if (auto v = nm.scalar("yecr")) M.yecr = to_logical(*v);
    if (auto v = nm.scalar("ystkmp")) M.ystkmp = to_logical(*v);
    if (auto v = nm.scalar("yrcmp")) M.yrcmp = to_logical(*v);
    if (auto v = nm.scalar("y_secd")) M.y_secd = to_logical(*v);
    if (auto v = nm.scalar("title")) {
      M.title = *v;
      M.title.resize(20, ' ');
    }
    if (auto v = nm.scalar("yspipro"); v && to_logical(*v))
      throw Error("yspipro (spin-adapted lists) is not supported");
    std::printf(" seuil de selection %10.5f\n nombre maximal de determinants %10d\n", M.tau, kNdimh);
    read_unit40(M);
    build_list(M);
    const int n = (int)M.ne.size();
    std::printf(" determinants engendres\n%12d\n", n);
    if (n > kNdimh) throw Error("stop 99: more than 10000000 determinants");
    if (n == 0) throw Error("no determinant read from unit 60");
    // moy.f:79-104: units 64 and 61
    {
      const int ii = M.nd[n - 1] + M.ne[n - 1] + 1;
      std::FILE* f64 = std::fopen(M.f64.c_str(), "wb");
      if (!f64) throw Error("cannot write " + M.f64);
      RecWriter w;
      w.put<int32_t>(n);
      w.put<int32_t>(ii);
      w.put<int32_t>(2 * M.norb);
      w.put<uint8_t>(0);
      for (int i = 0; i < n; ++i) {
        w.put<int32_t>(M.ne[i]);
        w.put<int32_t>(M.nd[i]);
      }
      for (int i = 0; i < ii; ++i) {
        w.put<int32_t>(i < (int)M.trou.size() ? M.trou[i] : 0);
        w.put<int32_t>(i < (int)M.part.size() ? M.part[i] : 0);
      }
      for (int i = 1; i <= 2 * M.norb + 1; ++i) w.put<int32_t>(i <= 2 * M.norb ? (i - 1) % M.norb + 1 : 0);
      for (int i = 1; i <= 2 * M.norb + 1; ++i) w.put<int32_t>(i <= 2 * M.norb ? (i > M.norb ? 1 : 0) : 0);
      w.flush(f64);
      std::fclose(f64);
      std::FILE* f61 = std::fopen(M.f61.c_str(), "wb");
      if (!f61) throw Error("cannot write " + M.f61);
      for (int i = 0; i < n; ++i) {
        RecWriter a;
        a.put<int32_t>(M.ne[i]);
        a.flush(f61);
        if (M.ne[i] != 0) {
          RecWriter b;
          for (int j = 0; j < M.ne[i]; ++j) b.put<int32_t>(M.trou[M.nd[i] + j]);
          for (int j = 0; j < M.ne[i]; ++j) b.put<int32_t>(M.part[M.nd[i] + j]);
          b.flush(f61);
        }
      }
      std::fclose(f61);
    }
    if (M.yrcmp) return 0;  // moy.f:106-107
    // the pairs on the GPU
    cipsi_dims d{};
    d.norb = M.norb;
    d.noca = M.noca;
    d.nsym = M.nsym;
    d.isym = M.isym > 0 ? M.isym : 1;
    d.isz = 0;
    d.metat = 1;
    d.ncf = n;
    auto chk = [&](int code, const char* what) {
      if (code) throw Error(std::string(what) + ": " + cipsi_last_error(ctx));
    };
    chk(cipsi_ctx_create(&ctx, &d, device), "cipsi_ctx_create");
    chk(cipsi_set_integrals(ctx, M.itsym.data(), M.its.data(), M.F.data(), M.J.data(), M.K.data(), M.ij0.data(),
                            M.ntttt.data(), M.eri.data(), (int64_t)M.eri.size()),
        "cipsi_set_integrals");
    {
      std::vector<uint8_t> zero8(n, 0);
      std::vector<int32_t> zero32(n, 0);
      chk(cipsi_set_space(ctx, M.ne.data(), M.nd.data(), M.trou.data(), M.part.data(), (int64_t)M.trou.size(),
                          zero8.data(), zero8.data(), zero32.data(), zero8.data()),
          "cipsi_set_space");
    }
    int64_t npairs = 0;
    chk(cipsi_hamiltonian_build(ctx, M.F.data(), M.y_secd ? M.ndims : -1, &npairs), "cipsi_hamiltonian_build");
    const double h_ms = cipsi_hamiltonian_ms(ctx);
    // diagonal (moy.f:185-190) and unit 1, rows in chunks of at most ~32 M pairs
    std::vector<double> stefen(n), stefmp(n);
    for (int i = 0; i < n; ++i) {
      stefen[i] = hdig(M, i);
      stefmp[i] = hmp(M, i);
    }
    Morue mo(M, stefen, stefmp);
    Unit1Writer u1;
    u1.f = std::fopen(M.f01.c_str(), "wb");
    if (!u1.f) throw Error("cannot write " + M.f01);
    if (M.ndims != n) u1.morue = &mo;
    long long nhntd = 0, nhij = 0;
    std::vector<int64_t> rowptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    const long long kChunkPairs = 32ll << 20;
    for (int r0 = 0; r0 < n;) {
      // rows r0 .. r1-1 whose pairs fit the chunk (at least one row)
      int r1 = r0 + 1;
      {
        std::vector<int64_t> one(2);
        chk(cipsi_hamiltonian_get(ctx, r0, 1, one.data(), nullptr, nullptr), "cipsi_hamiltonian_get");
        long long acc = one[1];
        int step = 1;
        while (r1 < n) {
          const int nr = std::min(step, n - r1);
          std::vector<int64_t> rp((size_t)nr + 1);
          chk(cipsi_hamiltonian_get(ctx, r1, nr, rp.data(), nullptr, nullptr), "cipsi_hamiltonian_get");
          if (acc + rp[nr] > kChunkPairs) break;
          acc += rp[nr];
          r1 += nr;
          step = std::min(step * 2, 65536);
        }
      }
      const int nr = r1 - r0;
      rowptr.resize((size_t)nr + 1);
      chk(cipsi_hamiltonian_get(ctx, r0, nr, rowptr.data(), nullptr, nullptr), "cipsi_hamiltonian_get");
      col.resize((size_t)std::max<int64_t>(rowptr[nr], 1));
      val.resize((size_t)std::max<int64_t>(rowptr[nr], 1));
      chk(cipsi_hamiltonian_get(ctx, r0, nr, rowptr.data(), col.data(), val.data()), "cipsi_hamiltonian_get");
      for (int q = 0; q < nr; ++q) {
        const int i = r0 + q;
        for (int64_t t = rowptr[q]; t < rowptr[q + 1]; ++t) {
          ++nhntd;
          if (std::fabs(val[t]) < 1.0e-10) continue;
          ++nhij;
          u1.add(i + 1, col[t] + 1, val[t]);
        }
        ++nhntd;
        ++nhij;
        u1.add(i + 1, i + 1, stefen[i] * 0.5);
      }
      r0 = r1;
    }
    u1.finish();
    std::fclose(u1.f);
    cipsi_ctx_destroy(ctx);
    ctx = nullptr;
    if (u1.nbuf == 0) std::printf(" **** attention le dernier buffer sur 1 ne contient aucun element\n");
    std::printf(" *** fin de la construction de h ***\n appels a hntd %10lld elements stockes sur 1 %10lld\n", nhntd,
                nhij);
    if (M.ystkmp) {  // moy.f:200-208
      std::FILE* f63 = std::fopen(M.f63.c_str(), "wb");
      if (!f63) throw Error("cannot write " + M.f63);
      RecWriter w;
      for (double x : stefmp) w.put<double>(x);
      w.flush(f63);
      std::fclose(f63);
    }
    // morue.f: unit 33 (when S does not cover the list) and the fourth
    // unit-4 record, which replaces whatever followed the third (morue.f
    // 8300; its last word, ny, is never set in morue and is written as 0)
    const int mt = M.metat;
    if (M.ndims != n) {
      std::vector<double> x(mt);
      for (int m = 0; m < mt; ++m) x[m] = mo.hefmp[(m + 1) * (m + 2) / 2 - 1];
      stkener(M, "moyens mbp " + M.title, x);
      for (int m = 0; m < mt; ++m) x[m] = mo.hefen[(m + 1) * (m + 2) / 2 - 1];
      stkener(M, "moyens envp" + M.title, x);
      for (int m = 0; m < mt; ++m) x[m] = mo.hefenb[(m + 1) * (m + 2) / 2 - 1];
      stkener(M, "moyens enb " + M.title, x);
    }
    {
      std::ifstream f4(M.f04, std::ios::binary);
      long long keep = 0;
      for (int q = 0; q < 3; ++q) {
        int32_t a = 0, b = 0;
        if (!f4.read(reinterpret_cast<char*>(&a), 4) || a < 0) throw Error("unit 4: fewer than three records");
        f4.seekg(a, std::ios::cur);
        if (!f4.read(reinterpret_cast<char*>(&b), 4) || b != a) throw Error("unit 4: fewer than three records");
        keep += 8 + (long long)a;
      }
      f4.close();
      if (truncate(M.f04.c_str(), (off_t)keep) != 0) throw Error("cannot truncate " + M.f04);
      std::FILE* fo = std::fopen(M.f04.c_str(), "ab");
      if (!fo) throw Error("cannot append to " + M.f04);
      RecWriter w;
      for (double v : mo.hefmp) w.put<double>(v);
      for (double v : mo.hefen) w.put<double>(v);
      for (double v : mo.hefenb) w.put<double>(v);
      w.put<int32_t>(0);
      w.flush(fo);
      std::fclose(fo);
    }
    std::fflush(stdout);
    if (json_path) {
      std::ofstream j(json_path);
      j << "{\n  \"ncf\": " << n << ", \"ndims\": " << M.ndims << ", \"metat\": " << mt << ", \"norb\": " << M.norb
        << ",\n  \"nhntd\": " << nhntd << ", \"nhij\": " << nhij << ", \"unit1_records\": " << u1.records
        << ",\n  \"pairs\": " << npairs << ", \"hbuild_ms\": " << h_ms << ",\n";
      j << "  \"hefmp\": " << json_array(mo.hefmp) << ",\n  \"hefen\": " << json_array(mo.hefen)
        << ",\n  \"hefenb\": " << json_array(mo.hefenb) << ",\n";
      j << "  \"wall_s\": " << std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count()
        << ", \"variant\": \"moy\"\n}\n";
    }
    return 0;
  } catch (const std::exception& ex) {
    seterr(errbuf, errlen, ex.what());
    if (ctx) cipsi_ctx_destroy(ctx);
    return CIPSI_ERR_ARG;
  }
}
