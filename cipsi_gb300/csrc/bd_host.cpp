// bd_host.cpp -- host side of the GPU drop-in for bd.exe: the lowest
// eigenpairs of the CI matrix that moy wrote to unit 1, for the next
// perturbation run.
//
// Reads what the reference reads (namelists &bdfil and &option on standard
// input; the first two records of unit 4 for metat, the model-space size
// ncper and escf; unit 1 mat) and writes what it writes: the 'energies
// var.' record of unit 33 (the eigenvalues, bd/stkener.f), unit 59 bdvec
// with the eigenvectors and the total energies (qwvec), unit 55 with the
// vectors' components (qws), and the listing lines the Autocip driver
// reads (' ncf,netat,ncper,iget' then the values, bd/storic.f:22-26).
// The eigenpairs come from cipsi_davidson (davidson.cu): a block Davidson
// iteration on the GPU, converged to a residual norm of 1e-8 Eh for every
// root; bd itself stops when its last correction's weight falls below
// 10 * test (bd/bigdia.f:402-411), so its vectors carry that tolerance.
//
// Followed sources: bd/bd.f (defaults 24-62, unit 4 58-61, the size of the
// matrix from unit 1 67-77, &option 84-115), bd/openf.f, bd/storic.f,
// bd/bigdia.f (outputs 60-75 and 385-433), bd/wvec.f (unit 55), bd/getmat.f
// (H = L + L^T with the diagonal stored as half its value).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cipsi_gb300.h"
#include "host_io.h"

namespace {

using namespace cipsi_host;

constexpr int kLsize = 8192;  // bd/bd.prm lsize

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

extern "C" int cipsi_bd_main(const char* workdir, const char* stdin_path, const char* json_path, int32_t device,
                             char* errbuf, int32_t errlen) {
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
    // openf.f
    const std::set<std::string> bdfil = {"prefix", "f04", "f041", "det_spin", "det_spin1", "det_cl", "mat",
                                         "det_cl1", "mat1", "ener", "ener1", "bdvec", "bdvec1"};
    Namelist cf = parse_namelist(text, "bdfil", bdfil);
    const std::string f01 = unit_file(cf, "mat", "mat1", "mat", dir);
    const std::string f04 = unit_file(cf, "f04", "f041", "f04", dir);
    const std::string f33 = unit_file(cf, "ener", "ener1", "ener", dir);
    const std::string f59 = unit_file(cf, "bdvec", "bdvec1", "bdvec", dir);
    const std::string f55 = dir + "/fort.55";  // unit 55 is not named by openf.f
    // bd.f:24-62: defaults, then metat, ncper and escf from unit 4 (a short
    // or missing unit 4 leaves what was read, bd.f:58-61 end=/err=7777)
    int metat = 1, ncper = 1, niter = 50;
    double test = 1.0e-4, escf = 0.0;
    bool qwvec = false, qws = false, qwb = false;
    std::string title = "                    ";
    {
      std::vector<Record> r4;
      try {
        r4 = read_records(f04);
      } catch (const Error&) {
      }
      if (!r4.empty() && r4[0].b.size() >= 20) {
        Record& a = r4[0];
        for (int q = 0; q < 3; ++q) (void)a.get<int32_t>();
        metat = a.get<int32_t>();
        ncper = a.get<int32_t>();
        const int nbr = metat * (metat + 1) / 2;
        if (r4.size() >= 2 && r4[1].b.size() >= (size_t)(nbr + 1) * 8) {
          for (int q = 0; q < nbr; ++q) (void)r4[1].get<double>();
          escf = r4[1].get<double>();
        }
      }
    }
    std::printf(" energie de reference \n %24.16E\n", escf);
    // bd.f:67-77: the order of the matrix is the largest index on unit 1
    std::vector<int32_t> I, J;
    std::vector<double> V;
    int ncf = 0;
    for (auto& r : read_records(f01)) {
      if (r.b.size() != (size_t)kLsize * 16) throw Error("unit 1: record of unexpected length");
      const int32_t* it = reinterpret_cast<const int32_t*>(r.b.data());
      const int32_t* jt = it + kLsize;
      const double* vb = reinterpret_cast<const double*>(jt + kLsize);
      const int last = it[kLsize - 1] == -1 ? jt[kLsize - 1] : kLsize;
      if (last < 0 || last > kLsize) throw Error("unit 1: bad element count in the last record");
      for (int l = 0; l < last; ++l) {
        I.push_back(it[l]);
        J.push_back(jt[l]);
        V.push_back(vb[l]);
        ncf = std::max(ncf, std::max(it[l], jt[l]));
      }
      if (it[kLsize - 1] == -1) break;
    }
    std::printf(" dimension de la matrice d ic sur la file 1 %10d\n", ncf);
    // &option (bd.f:16-19, 84)
    const std::set<std::string> option = {"qnorm", "netat", "spert", "ind", "cold", "mbuf", "qwa", "qwb", "qrvec",
                                          "ncf", "ncper", "metat", "test", "niter", "ezer", "ites", "qwvec", "qhef",
                                          "seuil", "ntrsy", "qws", "qsuis", "qsuip", "qener", "njter", "qgiv",
                                          "qictot", "qsui04", "qdcple", "tvec", "title", "ityp"};
    Namelist op = parse_namelist(text, "option", option);
    if (!op.found) throw Error("erreur dans la namelist option");
    auto r1 = [&](const char* k, double& d) { if (auto v = op.scalar(k)) d = to_real(*v); };
    auto i1 = [&](const char* k, int& d) { if (auto v = op.scalar(k)) d = to_int(*v); };
    auto l1 = [&](const char* k, bool& d) { if (auto v = op.scalar(k)) d = to_logical(*v); };
    i1("ncf", ncf);
    i1("ncper", ncper);
    i1("metat", metat);
    i1("niter", niter);
    r1("test", test);
    l1("qwvec", qwvec);
    l1("qws", qws);
    l1("qwb", qwb);
    if (auto v = op.scalar("title")) {
      title = *v;
      title.resize(20, ' ');
    }
    for (const char* k : {"qnorm", "qrvec", "qhef", "qdcple"}) {
      bool on = false;
      l1(k, on);
      if (on) throw Error(std::string(k) + " is not supported");
    }
    for (const char* k : {"ind", "cold", "netat", "ites"})
      if (op.has(k)) throw Error(std::string(k) + " given in &option is not supported");
    if (metat < 1 || metat > 8) throw Error("metat must be in [1, 8]");
    if (ncf < 1) throw Error("no element on unit 1");
    if (metat > ncf) throw Error("more roots than determinants");
    if (ncper > 2500) throw Error(" matrice de depart trop grande: diminuer ncper");
    // bd.f:105-115 with ites = 1: every root is computed (netat = metat)
    const int netat = metat;
    if (ncper > ncf) ncper = ncf;  // storic.f:21
    std::printf(" ncf,netat,ncper,iget\n %11d %11d %11d %11d\n", ncf, netat, ncper, 1);
    std::vector<double> ev(netat), vec((size_t)ncf * netat), res(netat);
    int iters = 0;
    char derr[512] = {0};
    const auto td0 = std::chrono::steady_clock::now();
    const int rc = cipsi_davidson(ncf, (int64_t)V.size(), I.data(), J.data(), V.data(), netat, 1.0e-8,
                                  std::max(niter, 200), device, ev.data(), vec.data(), &iters, res.data(), derr,
                                  (int32_t)sizeof derr);
    const double dav_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - td0).count();
    if (rc != 0) throw Error(derr);
    std::printf(" ref space energies");
    for (double e : ev) std::printf(" %14.6f", e);
    std::printf("\n");
    // bigdia.f:421-428 / 40-45: the eigenvalues on unit 33
    {
      std::FILE* f = std::fopen(f33.c_str(), "ab");
      if (!f) throw Error("cannot append to " + f33);
      std::string typ = "energies var." + title;
      typ.resize(40, ' ');
      RecWriter w;
      w.put_bytes(typ.data(), 40);
      for (double e : ev) w.put<double>(e);
      w.flush(f);
      std::fclose(f);
      std::printf(" *************************************\n %s stockee sur la file 33", typ.c_str());
      for (double e : ev) std::printf(" %24.16E", e);
      std::printf("\n *************************************\n");
    }
    // the norms in S (the first ncper determinants) and in the whole space
    // (wvec.f:58-70, printed with qwb or qws)
    if (qwb || qws) {
      std::printf(" ***  norme des etats ***\n etat       norme dans S      norme total\n");
      for (int m = 0; m < netat; ++m) {
        double ns = 0.0, nt = 0.0;
        for (int i = 0; i < ncf; ++i) {
          const double x = vec[(size_t)m * ncf + i] * vec[(size_t)m * ncf + i];
          nt += x;
          if (i < ncper) ns += x;
        }
        std::printf(" %3d    %15.8f  %15.8f\n", m + 1, ns, nt);
      }
    }
    // unit 55 (qws): the Davidson branch writes each vector's first ncper
    // components (wvec.f:73), the direct one (ncper >= ncf - metat) the
    // whole vectors (bigdia.f:69)
    if (qws) {
      const bool direct = ncper >= ncf - metat;
      std::FILE* f = std::fopen(f55.c_str(), "wb");
      if (!f) throw Error("cannot write " + f55);
      RecWriter w;
      w.put<int32_t>(ncper);
      w.put<int32_t>(netat);
      for (int m = 0; m < netat; ++m)
        for (int i = 0; i < (direct ? ncf : ncper); ++i) w.put<double>(vec[(size_t)m * ncf + i]);
      for (double e : ev) w.put<double>(e);
      w.flush(f);
      std::fclose(f);
    }
    // unit 59 (qwvec): ncf, netat, the vectors, the total energies
    // (bigdia.f:429-431)
    if (qwvec) {
      std::FILE* f = std::fopen(f59.c_str(), "wb");
      if (!f) throw Error("cannot write " + f59);
      RecWriter w;
      w.put<int32_t>(ncf);
      w.put<int32_t>(netat);
      for (double x : vec) w.put<double>(x);
      for (double e : ev) w.put<double>(e + escf);
      w.flush(f);
      std::fclose(f);
    }
    std::fflush(stdout);
    if (json_path) {
      std::ofstream j(json_path);
      j << "{\n  \"ncf\": " << ncf << ", \"netat\": " << netat << ", \"ncper\": " << ncper
        << ", \"elements\": " << V.size() << ",\n  \"eigenvalues\": " << json_array(ev)
        << ",\n  \"residuals\": " << json_array(res) << ",\n  \"escf\": " << json_array({escf})
        << ",\n  \"iterations\": " << iters << ", \"davidson_s\": " << dav_s << ",\n  \"wall_s\": "
        << std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() << "\n}\n";
    }
    return 0;
  } catch (const std::exception& ex) {
    seterr(errbuf, errlen, ex.what());
    return CIPSI_ERR_ARG;
  }
}
