/*
 * cipsi_ref.c -- CPU oracle for the CIPSI second-order perturbation /
 * selection step ("cip" and "cipsym" executables of the Toulouse CIPSI chain).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a line-by-line C restatement of the
 * reference Fortran path so that the GPU engine can be checked against it.
 * Only tests/, the smoke check and bench.py's cpu_baseline leg may build or run
 * it; the product never links it.
 *
 * Parity status: UNPINNED by the reference itself.  The reference ships no
 * tests, fixtures or golden vectors, and its executables (ifort + MKL builds)
 * cannot run without the Intel runtime, and no Fortran compiler is available,
 * so this restatement cannot be cross-checked against cip.exe output.  It is
 * instead cross-checked against an independent brute-force model
 * (tests/brute_force.py) on small systems: the perturber set, spin-flip
 * weights and couplings (tests/test_oracle_semantics.py), and the E2 sums,
 * norms, ietat, histogram, unit-60 values, dpivot and selected set, under
 * several option sets (tests/test_oracle_e2.py).
 *
 * Followed sources (paths inside the reference project):
 *   CIPSI_sources/cip/cip.f      main flow 50-242, outputs 243-425
 *   CIPSI_sources/cip/openf.f    &cipfil, unit names
 *   CIPSI_sources/cip/deter.f    defaults 78-227, S build with spin-flip
 *                                partners 478-567
 *   CIPSI_sources/cip/transf.f   sort / validate / dedup of one determinant
 *   CIPSI_sources/cip/lec60.f    reading S from unit 60
 *   CIPSI_sources/cipsym/cas.f   complete active space (lecdet=4)
 *   CIPSI_sources/cipsym/shell.f, cip.f:200-236   the run that only writes
 *                                S (ityper<0): energy order, units 4 and 60
 *   CIPSI_sources/cip/ijkf.f, reijkl.f, rdener.f, ic001.f:44-76 (lecdet=5),
 *   CIPSI_sources/cip/brdnee.f:299-365 (degen, the rotation of degenerate roots)
 *   CIPSI_sources/cip/faifoc.f, hmp.f, hdig.f, hntd.f, ai.f
 *   CIPSI_sources/cip/pertu.f, igene.f, cotra.f, pert1.f, diexcit.f,
 *   CIPSI_sources/cip/isto.f, pie.f, stkener.f
 *   CIPSI_sources/cipsym/pie.f, pert1.f:244, diexcit.f:446, cip.f:226-254,
 *   CIPSI_sources/cipsym/ic001.f:179 (all determinants are generators)
 *   CIPSI_sources/cip/ic001.f:81-131 (lecdet != 5: H over S and its lowest
 *                                roots, here by Jacobi rotations)
 *   CIPSI_sources/moy/*.f        the Hamiltonian over unit 60 (--moy)
 *
 * Arrays are 1-based (index 0 unused) to keep the restatement checkable
 * against the Fortran line by line.
 *
 * Not restated (rejected with an error): lecdet=1 (card input), ybrd (QDPT
 * effective Hamiltonian), yion (excitation to infinity), iord or ygen given
 * in the namelist.
 */
#define _GNU_SOURCE
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

/* ---------------------------------------------------------------- utils */
static void die(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  fprintf(stderr, "cipsi_ref: ");
  vfprintf(stderr, fmt, ap);
  fprintf(stderr, "\n");
  va_end(ap);
  exit(2);
}
static void* xcalloc(size_t n, size_t s) {
  void* p = calloc(n ? n : 1, s ? s : 1);
  if (!p) die("out of memory (%zu x %zu)", n, s);
  return p;
}

/* ------------------------------------------- Fortran unformatted records */
typedef struct {
  unsigned char* b;
  int32_t len;
  int32_t pos;
} rec_t;

static int rec_read(FILE* f, rec_t* r) {
  int32_t n1, n2;
  if (fread(&n1, 4, 1, f) != 1) return 0;
  free(r->b);
  r->b = (unsigned char*)xcalloc((size_t)n1 + 8, 1);
  if (n1 && fread(r->b, 1, (size_t)n1, f) != (size_t)n1) die("truncated record");
  if (fread(&n2, 4, 1, f) != 1 || n2 != n1) die("bad record marker");
  r->len = n1;
  r->pos = 0;
  return 1;
}
static int32_t rec_i4(rec_t* r) {
  int32_t v;
  if (r->pos + 4 > r->len) die("record too short (i4)");
  memcpy(&v, r->b + r->pos, 4);
  r->pos += 4;
  return v;
}
static int16_t rec_i2(rec_t* r) {
  int16_t v;
  if (r->pos + 2 > r->len) die("record too short (i2)");
  memcpy(&v, r->b + r->pos, 2);
  r->pos += 2;
  return v;
}
static double rec_r8(rec_t* r) {
  double v;
  if (r->pos + 8 > r->len) die("record too short (r8)");
  memcpy(&v, r->b + r->pos, 8);
  r->pos += 8;
  return v;
}
static float rec_r4(rec_t* r) {
  float v;
  if (r->pos + 4 > r->len) die("record too short (r4)");
  memcpy(&v, r->b + r->pos, 4);
  r->pos += 4;
  return v;
}
static int rec_l1(rec_t* r) {
  if (r->pos + 1 > r->len) die("record too short (l1)");
  return r->b[r->pos++] != 0;
}

typedef struct {
  unsigned char* b;
  size_t len, cap;
} wbuf_t;
static void wb_put(wbuf_t* w, const void* p, size_t n) {
  if (w->len + n > w->cap) {
    w->cap = (w->len + n) * 2 + 64;
    w->b = (unsigned char*)realloc(w->b, w->cap);
    if (!w->b) die("oom");
  }
  memcpy(w->b + w->len, p, n);
  w->len += n;
}
static void wb_i4(wbuf_t* w, int32_t v) { wb_put(w, &v, 4); }
static void wb_r8(wbuf_t* w, double v) { wb_put(w, &v, 8); }
static void wb_flush(FILE* f, wbuf_t* w) {
  int32_t n = (int32_t)w->len;
  fwrite(&n, 4, 1, f);
  if (n) fwrite(w->b, 1, w->len, f);
  fwrite(&n, 4, 1, f);
  w->len = 0;
}

/* ------------------------------------------------------ namelist parsing */
/* Fortran namelist reader: "&group" up to "&end" or "/"; "name = values"
   (names in any case) with values separated by commas and/or blanks, "r*c"
   for r copies of c, "r*" or nothing between two commas for a null value
   (the element keeps its value), "name(i) = values" from element i on, "!"
   comments to the end of the line.  An item holds its elements 1..nval
   (val[i-1], NULL where not assigned); a name outside `names` is an error,
   as it is for the Fortran runtime (deter.f:222 -> 9500). */
typedef struct {
  char key[64];
  int nval;
  char** val;
} nlitem_t;
typedef struct {
  int n;
  nlitem_t it[128];
} nlgroup_t;

static char* g_stdin_text = NULL;

static void lower(char* s) {
  for (; *s; s++) *s = (char)tolower((unsigned char)*s);
}

static nlitem_t* nl_get(nlgroup_t* g, const char* key) {
  for (int i = 0; i < g->n; i++)
    if (strcasecmp(g->it[i].key, key) == 0) return &g->it[i];
  return NULL;
}

static void nl_put(nlitem_t* it, int idx, const char* v) {
  if (idx > it->nval) {
    it->val = (char**)realloc(it->val, sizeof(char*) * (size_t)idx);
    for (int i = it->nval; i < idx; i++) it->val[i] = NULL;
    it->nval = idx;
  }
  if (v) {
    free(it->val[idx - 1]);
    it->val[idx - 1] = strdup(v);
  }
}

static int nl_parse(const char* group, nlgroup_t* g, const char* const* names) {
  memset(g, 0, sizeof(*g));
  const char* t = g_stdin_text;
  size_t gl = strlen(group);
  const char* p = NULL;
  for (const char* q = t; *q; q++) {
    if (*q == '&' && strncasecmp(q + 1, group, gl) == 0 &&
        !isalnum((unsigned char)q[1 + gl]) && q[1 + gl] != '_') {
      p = q + 1 + gl;
      break;
    }
  }
  if (!p) return 0;
  char tok[4096];
  nlitem_t* cur = NULL;
  int idx = 1, need_sep = 0;
  while (*p) {
    if (isspace((unsigned char)*p)) { p++; continue; }
    if (*p == '!') {
      while (*p && *p != '\n') p++;
      continue;
    }
    if (*p == '/' || *p == '&') break; /* &end or next group */
    if (*p == ',') {
      if (!need_sep && cur) nl_put(cur, idx++, NULL); /* null value */
      need_sep = 0;
      p++;
      continue;
    }
    int n = 0, quoted = 0;
    if (*p == '\'' || *p == '"') {
      char qc = *p++;
      quoted = 1;
      while (*p && n < 4095) {
        if (*p == qc) {
          if (p[1] == qc) { tok[n++] = qc; p += 2; continue; }
          p++;
          break;
        }
        tok[n++] = *p++;
      }
      tok[n] = 0;
    } else {
      while (*p && !isspace((unsigned char)*p) && *p != ',' && *p != '=' && *p != '/' && *p != '!' &&
             n < 4095)
        tok[n++] = *p++;
      tok[n] = 0;
    }
    const char* r = p;
    while (*r && isspace((unsigned char)*r)) r++;
    if (!quoted && *r == '=') {
      p = r + 1;
      lower(tok);
      idx = 1;
      char* lp = strchr(tok, '(');
      if (lp) {
        idx = atoi(lp + 1);
        *lp = 0;
        if (idx < 1) die("erreur dans la namelist %s: bad subscript", group);
      }
      int known = 0;
      for (const char* const* nm = names; *nm; nm++)
        if (!strcmp(*nm, tok)) known = 1;
      if (!known) die("erreur dans la namelist %s: unknown name %s", group, tok);
      cur = nl_get(g, tok);
      if (!cur) {
        if (g->n >= 128) die("namelist too long");
        cur = &g->it[g->n++];
        snprintf(cur->key, sizeof cur->key, "%.60s", tok);
      }
      need_sep = 0;
      continue;
    }
    if (!cur) die("namelist &%s: value without key: %s", group, tok);
    char* star = quoted ? NULL : strchr(tok, '*');
    int digits = star && star > tok;
    for (char* c = tok; digits && c < star; c++)
      if (!isdigit((unsigned char)*c)) digits = 0;
    if (digits) { /* r*c or r* */
      int rep = atoi(tok);
      char* c = star + 1;
      size_t cl = strlen(c);
      if (cl >= 2 && (c[0] == '\'' || c[0] == '"') && c[cl - 1] == c[0]) {
        c[cl - 1] = 0;
        c++;
      }
      for (int q = 0; q < rep; q++) nl_put(cur, idx++, *c ? c : NULL);
    } else {
      nl_put(cur, idx++, (quoted && !n) ? " " : tok);
    }
    need_sep = 1;
  }
  return 1;
}
static double nl_real(const char* s) {
  char b[128], *end;
  snprintf(b, sizeof b, "%s", s);
  for (char* c = b; *c; c++)
    if (*c == 'd' || *c == 'D') *c = 'e';
  double v = strtod(b, &end);
  if (end == b || *end) die("erreur dans la namelist icinp: bad real value %s", s);
  return v;
}
static int nl_integer(const char* s) {
  char* end;
  long v = strtol(s, &end, 10);
  if (end == s || *end) die("erreur dans la namelist icinp: bad integer value %s", s);
  return (int)v;
}
static int nl_logical(const char* s) {
  while (*s == '.') s++;
  if (!*s || !strchr("tTfF", *s)) die("erreur dans la namelist icinp: bad logical value %s", s);
  return *s == 't' || *s == 'T';
}
/* the value of a scalar, or NULL */
static const char* nl_scalar(nlgroup_t* g, const char* k) {
  nlitem_t* it = nl_get(g, k);
  if (!it || !it->nval) return NULL;
  if (it->nval > 1) die("erreur dans la namelist: too many values for %s", k);
  return it->val[0];
}
static void nl_set_int(nlgroup_t* g, const char* k, int* dst) {
  const char* v = nl_scalar(g, k);
  if (v) *dst = nl_integer(v);
}
static void nl_set_real(nlgroup_t* g, const char* k, double* dst) {
  const char* v = nl_scalar(g, k);
  if (v) *dst = nl_real(v);
}
static void nl_set_log(nlgroup_t* g, const char* k, int* dst) {
  const char* v = nl_scalar(g, k);
  if (v) *dst = nl_logical(v);
}
/* array elements 1..bound: dst[i-1] for the assigned i <= napply */
static void nl_set_real_arr(nlgroup_t* g, const char* k, double* dst, int napply, int bound) {
  nlitem_t* it = nl_get(g, k);
  if (!it) return;
  if (it->nval > bound) die("erreur dans la namelist: %s has more than %d elements", k, bound);
  for (int i = 0; i < it->nval && i < napply; i++)
    if (it->val[i]) dst[i] = nl_real(it->val[i]);
}
static void nl_set_int_arr(nlgroup_t* g, const char* k, int* dst, int napply, int bound) {
  nlitem_t* it = nl_get(g, k);
  if (!it) return;
  if (it->nval > bound) die("erreur dans la namelist: %s has more than %d elements", k, bound);
  for (int i = 0; i < it->nval && i < napply; i++)
    if (it->val[i]) dst[i] = nl_integer(it->val[i]);
}

/* ------------------------------------------------------------ the state */
/* COMMON /cipsi/ */
/* dimension of nblock / nstart in the reference's parameter file
   (pshf.prm ndetz): unit 4 carries both arrays in full */
#define UNIT4_NDETZ 500000
static double escf, test, teseff, tdet, twdet, coeff, tau;
static int ndiag, norb, mnorb, noca, nocb, noc1, noc2, igela, igelb, ncf, nsym, isym, isz,
    ntrsy, metat, lecdet, maxdet, ityper, iselec, nclass, ninact;
static int yprt, yion, ypertu, ybrd, yen, ywvi, ywvf, ytoul, ystkic, ywdeg, ymoyen, yselm,
    ysele, ydp, yreduc, ytocom;
static int g_sym_variant = 0; /* 1 = cipsym behaviour */

/* /spo/ */
static double* fdiag; /* 2*norb */
static double* hdiag; /* ncf */
static double* tocom; /* 2*norb */
static int *ispin, *iorb, *itsym; /* spin orbitals 1..mnorb */
static int its[24][24];
static unsigned char *yoc, *yocs; /* 1..mnorb */
static unsigned char* ygen;       /* 1..ncf */
static unsigned char* yocd_;      /* (mnorb+1) x (ncf+2) */
static int yocd_ld;
#define YOCD(so, k) yocd_[(size_t)(k) * (size_t)yocd_ld + (size_t)(so)]
static int *ne, *nd, *trou, *part; /* dets 1..ncf+1, trou/part 1..ntp */
static int ntp_cap;
static int numero[64];
/* /degene/ */
static int *nesp, *nespo, *isytr1; /* isytr(.,1) spin flip map */
static unsigned char *ysaut, *yef1;
/* /ic/ */
static double* c; /* metat*ncf column-major per root */
static double e[64], eb[64], e2b[64], emp[64], teste[64], e2mp[64], e2vp[64], psimp[64],
    psivp[64], taum[64];
static double dpivot;
static long long ietat;
/* first-order rounding-propagation bound of each E2 sum (not in cip): the
   sum over perturbers of |term| * (2*kb + kd), kb = 16u*sum|H c|/|b|,
   kd = 16u*(|E0| + sum of |diagonal terms|)/|denominator| */
static double cond_mp[64], cond_vp[64], cond_b[64];
/* instrumentation (not in cip): the same E2 terms summed with an error-free
   two-sum (value + accumulated rounding errors), to separate the serial
   sum's own rounding from differences of the terms */
static double ks_mp[64], kc_mp[64], ks_vp[64], kc_vp[64], ks_b[64], kc_b[64];
static void comp_add(double* sum, double* err, double t) {
  const double a = *sum + t;
  const double bp = a - *sum;
  *err += (*sum - (a - bp)) + (t - bp);
  *sum = a;
}
#define U16 (16.0 * 1.1102230246251565e-16)
static double* fmpb;
/* /hist/ */
static long long nom[11], nam[11][64];
static double aval[11], tabmp[11][64], tabvp[11][64], semp[64], sevp[64];
/* /orper/ */
static unsigned char* yorper; /* orbitals 1..norb */
/* /jkf/ */
static double *f_, *aj, *ak;
/* /ij1/, /bij/ */
static int16_t* ij0_; /* norb x norb, Fortran column-major ij0(i,j) */
#define IJ0(i, j) ij0_[((size_t)(j)-1) * (size_t)norb + ((size_t)(i)-1)]
static int ntttt[24];
static float* bijkl;
static long long ninte;
/* /det/ (pie) */
#define LUNGO 1000
static int det_m, det_n, det_idet[16 * LUNGO + 16], det_nex[LUNGO + 2];
static double det_v[LUNGO + 2], det_evp[LUNGO * 64 + 64];
static long long det_ntot;
static FILE* f60 = NULL;

/* instrumentation (not part of cip) */
static unsigned char* gen_mask = NULL; /* 1..ncf: 1 = run as generator */
static int run_pertu_ref = 1;          /* include pertu's kk=0 candidates */
static FILE* cand_log = NULL;
static long long n_processed = 0;      /* perturbers reaching the E2 loop */
static int cur_src = 0;                /* 0 pertu, 1 igene, 2 diexcit */
/* systematic sample (CPU timing only, --sample M with --plan): one pert1
   candidate in M, and one diexcit hole/particle quadruple in M, counted in
   enumeration order from samp_seq; residue samp_m is kept */
static long long samp_M = 0, samp_m = 0, samp_seq = 0;

static int noc_[3], igels_[3], norbs_[3]; /* equivalence (noca,noc(1)) etc. */

static int hf_noc; /* noc from unit 40 */
/* /activ/: the CAS of lecdet = 4 (numac(1..noac) active orbitals, nelac
   active electrons, nusym its symmetry, nemax its largest excitation) */
static int numac[520], noac, nusym, nelac, nemax;
static char title[64] = "                    ";

/* ------------------------------------------------------- ai (cip/ai.f) */
static double ai(int i, int j, int k, int l) {
  int ij, isy, kl, jsy;
  if (j >= i) {
    ij = IJ0(i, j);
    isy = (i == j) ? 1 : IJ0(j, i);
  } else {
    ij = IJ0(j, i);
    isy = IJ0(i, j);
  }
  if (l >= k) {
    kl = IJ0(k, l);
    jsy = (k == l) ? 1 : IJ0(l, k);
  } else {
    kl = IJ0(l, k);
    jsy = IJ0(k, l);
  }
  if (isy != jsy) return 0.0;
  long long ijkl;
  if (ij <= kl)
    ijkl = (long long)ij + ((long long)kl * kl - kl) / 2 + ntttt[isy] - 1;
  else
    ijkl = (long long)kl + ((long long)ij * ij - ij) / 2 + ntttt[isy] - 1;
  return (double)bijkl[ijkl];
}
static inline int num(int i) { return i * (i - 1) / 2; }

/* ------------------------------------------------------ hmp (cip/hmp.f) */
static double hmp(int iiii) {
  int nei = ne[iiii];
  if (nei == 0) return 0.0;
  int l1 = nd[iiii], l2 = l1 + nei;
  l1 = l1 + 1;
  double ac = 0.0;
  for (int l = l1; l <= l2; l++) ac = ac + fmpb[part[l]] - fmpb[trou[l]];
  return ac;
}

/* ---------------------------------------------------- hdig (cip/hdig.f) */
static double hdig(int iii) {
  int nei = ne[iii];
  if (nei == 0) return 0.0;
  int l1 = nd[iii], l2 = l1 + nei;
  l1 = l1 + 1;
  double ab = 0.0;
  for (int l = l1; l <= l2; l++) {
    int n1p = part[l], n1t = trou[l];
    ab = ab + fdiag[n1p] - fdiag[n1t];
    int ns1t = ispin[n1t], ns1p = ispin[n1p];
    n1t = iorb[n1t];
    n1p = iorb[n1p];
    for (int j = l1; j <= l; j++) {
      int n2t = trou[j], n2p = part[j];
      int ns2t = ispin[n2t], ns2p = ispin[n2p];
      n2t = iorb[n2t];
      n2p = iorb[n2p];
      int n12t, n12p;
      if (n2t > n1t)
        n12t = num(n2t) + n1t;
      else
        n12t = num(n1t) + n2t;
      if (n2p > n1p)
        n12p = num(n2p) + n1p;
      else
        n12p = num(n1p) + n2p;
      int n1tp = num(n2p) + n1t;
      int n2tp = num(n1p) + n2t;
      double ca = aj[n12t] + aj[n12p] - aj[n1tp] - aj[n2tp];
      if (ns1t == ns2t) ca = ca - ak[n12t];
      if (ns1p == ns2p) ca = ca - ak[n12p];
      if (ns1t == ns2p) ca = ca + ak[n1tp];
      if (ns1p == ns2t) ca = ca + ak[n2tp];
      if (j == l) ca = 0.5 * ca;
      ab = ab + ca;
    }
  }
  return ab;
}

/* sums of |terms| of hmp and hdig (for the rounding bound only) */
static double hmp_abs(int iiii) {
  double ac = 0.0;
  for (int l = nd[iiii] + 1; l <= nd[iiii] + ne[iiii]; l++) ac += fabs(fmpb[part[l]]) + fabs(fmpb[trou[l]]);
  return ac;
}
static double hdig_abs(int iii) {
  double ab = 0.0;
  int l1 = nd[iii] + 1, l2 = nd[iii] + ne[iii];
  for (int l = l1; l <= l2; l++) {
    ab += fabs(fdiag[part[l]]) + fabs(fdiag[trou[l]]);
    int n1t = iorb[trou[l]], n1p = iorb[part[l]];
    for (int j = l1; j <= l; j++) {
      int n2t = iorb[trou[j]], n2p = iorb[part[j]];
      int n12t = n2t > n1t ? num(n2t) + n1t : num(n1t) + n2t;
      int n12p = n2p > n1p ? num(n2p) + n1p : num(n1p) + n2p;
      ab += fabs(aj[n12t]) + fabs(aj[n12p]) + fabs(aj[num(n2p) + n1t]) + fabs(aj[num(n1p) + n2t]);
      ab += fabs(ak[n12t]) + fabs(ak[n12p]) + fabs(ak[num(n2p) + n1t]) + fabs(ak[num(n1p) + n2t]);
    }
  }
  return ab;
}

/* ---------------------------------------------------- hntd (cip/hntd.f) */
static double hntd(int ii, int jj) {
  int ita[24], itb[24], nv1[3], nv2[3], natu1[3], natu2[3];
  int kr, kl;
  if (ne[ii] - ne[jj] <= 0) {
    kr = jj;
    kl = ii;
  } else {
    kr = ii;
    kl = jj;
  }
  int ne1 = ne[kr];
  if (ne1 == 0) return 0.0; /* identity */
  int ne2 = ne[kl];
  int nbdif = ne1 - ne2;
  if (nbdif > 2) return 0.0;
  int nd1 = nd[kr], nd2 = nd[kl];
  for (int j = 1; j <= ne1; j++) {
    ita[j] = trou[j + nd1];
    ita[j + ne1] = part[j + nd1];
  }
  int ysig = 0;
  if (ne2 != 0) {
    for (int j = 1; j <= ne2; j++) {
      itb[j] = trou[j + nd2];
      itb[j + ne2] = part[j + nd2];
    }
    for (int k = 1; k <= 2; k++) {
      int k1 = (k - 1) * ne1, k2 = (k - 1) * ne2;
      for (int i = 1; i <= ne2; i++) {
        int nit1 = itb[k2 + i];
        int j1 = 1 + k1, j2 = ne1 + k1;
        int found = 0;
        for (int j = j1; j <= j2; j++) {
          int njt2 = ita[j];
          if (nit1 != njt2) continue;
          if (i != (j - k1)) {
            ita[j] = ita[i + k1];
            ita[i + k1] = njt2;
            ysig = !ysig;
          }
          found = 1;
          break;
        }
        if (found) continue;
        nbdif = nbdif + 1;
        if (nbdif > 2) return 0.0;
        nv1[nbdif] = nit1;
        natu1[nbdif] = k;
        natu2[nbdif] = i;
      }
    }
  }
  if (nbdif <= 0) return 0.0; /* identity */
  int nar = ne1 - ne2;
  if (nar > 0) {
    for (int i = 1; i <= nar; i++) {
      int net = ne1 + 1 - i;
      nv1[i] = ita[net];
      nv2[i] = ita[net + ne1];
    }
  }
  int nbar = nbdif - nar;
  if (nbar > 0) {
    for (int i = nar + 1; i <= nbdif; i++) {
      int k = natu1[i], ni = natu2[i], nu = nv1[i];
      nv2[i] = ita[ni + ne1 * (k - 1)];
      if (k == 2) continue;
      nv1[i] = nv2[i];
      nv2[i] = nu;
      ysig = !ysig;
    }
  }
  double ha = 0.0;
  int n1 = iorb[nv1[1]], n2 = iorb[nv2[1]];
  int ns1 = ispin[nv1[1]], ns2 = ispin[nv2[1]];
  int ncr = ysig ? -1 : 1;
  if (nbdif != 1) {
    int n3 = iorb[nv1[2]], n4 = iorb[nv2[2]];
    int ns4 = ispin[nv2[2]];
    if (ns1 == ns2) ha = ai(n1, n2, n3, n4);
    if (ns1 == ns4) ha = ha - ai(n1, n4, n3, n2);
  } else {
    int n12 = (n2 >= n1) ? num(n2) + n1 : num(n1) + n2;
    ha = f_[n12];
    for (int i = 1; i <= ne1; i++) {
      int np = iorb[ita[i]];
      int nsu = ispin[ita[i]];
      double aix = ai(n1, n2, np, np);
      ha = ha - aix;
      if (ns1 == nsu) ha = ha + ai(n1, np, n2, np);
      np = iorb[ita[i + ne1]];
      if (np > norb) continue;
      nsu = ispin[ita[i + ne1]];
      ha = ha + ai(n1, n2, np, np);
      if (ns1 == nsu) ha = ha - ai(n1, np, n2, np);
    }
  }
  return ha * ncr;
}

/* --------------------------------------------------- isto (cip/isto.f) */
static void isto(double val, const double* vil, int nespf, double* fmul) {
  if (val < teseff) return;
  int nc = nclass - 1;
  *fmul = *fmul + 1.0;
  int i;
  for (i = 1; i <= nc; i++)
    if (val < aval[i]) break;
  int cls = (i <= nc) ? i : nclass;
  nom[cls] = nom[cls] + 1 + nespf;
  for (int m = 1; m <= metat; m++) {
    if (vil[m] < teseff) continue;
    tabmp[cls][m] = tabmp[cls][m] + semp[m] * (*fmul);
    tabvp[cls][m] = tabvp[cls][m] + sevp[m] * (*fmul);
  }
  for (int m = 1; m <= metat; m++) {
    if (vil[m] < teseff) continue;
    for (i = 1; i <= nc; i++)
      if (vil[m] < aval[i]) break;
    int c2 = (i <= nc) ? i : nclass;
    nam[c2][m] = nam[c2][m] + nespf + 1;
  }
}

/* ----------------------------------------- pie / fine (cip/pie.f, cipsym) */
static void fine(void);
static void pie(int nec, const int* nts, const int* nps, double xam, const double* venvp) {
  if (nec > 8) die("degre d'excitation superieur a 8 (%d)", nec);
  for (int i = 1; i <= nec; i++) {
    det_idet[++det_m] = nts[i];
    det_idet[++det_m] = nps[i];
  }
  det_n++;
  det_ntot++;
  det_nex[det_n] = nec;
  det_v[det_n] = xam;
  if (g_sym_variant)
    for (int i = 1; i <= metat; i++) det_evp[(det_n - 1) * metat + i] = venvp ? venvp[i] : 0.0;
  if (det_n < LUNGO) return;
  fine();
}
static void fine(void) {
  if (det_n == 0) return;
  wbuf_t w = {0};
  wb_i4(&w, det_m);
  wb_i4(&w, det_n);
  for (int i = 1; i <= det_m; i++) wb_i4(&w, det_idet[i]);
  for (int i = 1; i <= det_n; i++) wb_i4(&w, det_nex[i]);
  for (int i = 1; i <= det_n; i++) wb_r8(&w, det_v[i]);
  if (g_sym_variant)
    for (int i = 1; i <= det_n * metat; i++) wb_r8(&w, det_evp[i]);
  wb_flush(f60, &w);
  free(w.b);
  det_m = 0;
  det_n = 0;
}

/* candidate log: one record per perturber reaching the E2 loop */
static void log_candidate(int kk, int nf, double xam, const double* him, double fmul, int nmul) {
  if (!cand_log) return;
  int nec = ne[nf];
  int h[16], p[16];
  for (int i = 1; i <= nec; i++) {
    h[i - 1] = trou[nd[nf] + i];
    p[i - 1] = part[nd[nf] + i];
  }
  /* sort ascending (set identity) */
  for (int a = 0; a < nec; a++)
    for (int b = a + 1; b < nec; b++) {
      if (h[b] < h[a]) { int t = h[a]; h[a] = h[b]; h[b] = t; }
      if (p[b] < p[a]) { int t = p[a]; p[a] = p[b]; p[b] = t; }
    }
  int32_t hdr[4] = {cur_src, kk, nec, nmul};
  fwrite(hdr, 4, 4, cand_log);
  int32_t hp[32];
  for (int i = 0; i < 16; i++) {
    hp[i] = i < nec ? h[i] : 0;
    hp[16 + i] = i < nec ? p[i] : 0;
  }
  fwrite(hp, 4, 32, cand_log);
  double d[2] = {xam, fmul};
  fwrite(d, 8, 2, cand_log);
  for (int m = 1; m <= metat; m++) fwrite(&him[m], 8, 1, cand_log);
}

/* ------------------------------------------------- pert1 (cip/pert1.f) */
static int* ikk_buf;
static double* stok_buf;

static void pert1(int kkmod, int nf) {
  if (samp_M > 1 && (samp_seq++ % samp_M) != samp_m) return;
  int nts[16], nps[16];
  double vil[64] = {0}, him[64], dmp[64], dvp[64], db[64], venvp[64];
  if (kkmod < 0) kkmod = 0;
  int kk = kkmod;
  int nec = ne[nf];
  int yf = (nec == 0);
  int ndf = nd[nf];
  double fmul = 0.0, fmulbr = 1.0;
  int nmul = 0, ybis = 0;
  if (!yf) {
    for (int i = 1; i <= nec; i++) {
      int nt = trou[ndf + i];
      nts[i] = nt;
      if (yoc[nt]) goto L200;
      yoc[nt] = 1;
      int np = part[ndf + i];
      nps[i] = np;
      if (yoc[np]) goto L200;
      yoc[np] = 1;
    }
  }
  if (yreduc) {
    if (nec == 0) goto L200;
    int ok = 0;
    for (int i = 1; i <= nec; i++) {
      int np = iorb[part[ndf + i]];
      if (yorper[np]) { ok = 1; break; }
    }
    if (!ok) goto L200;
  }
  kk = kkmod;
  /* owner test over generators j < kk (pert1.f:104-118) */
  for (int j = 1; j < kk; j++) {
    if (!ygen[j]) continue;
    int ndif = nec - ne[j];
    if (ndif > 2) continue;
    if (ne[j] == 0) goto L200;
    int nej = ne[j] + nd[j], ndj = nd[j] + 1;
    for (int i = ndj; i <= nej; i++) {
      if (!yoc[trou[i]]) ndif++;
      if (!yoc[part[i]]) ndif++;
    }
    if (ndif <= 2) goto L200;
  }
  {
    int ijune = 0;
    if (kk == 0) kk = 1;
    int lesp = 0;
    int nespf = nesp[kk];
    if (kkmod == 0) nespf = 0;
    int kkmax = kk + nespf;
    /* interaction scan j = kk..ncf (pert1.f:129-144) */
    for (int j = kk; j <= ncf; j++) {
      int ndif = nec - ne[j];
      if (ndif > 2) continue;
      if (ne[j] != 0) {
        int nej = ne[j] + nd[j], ndj = nd[j] + 1;
        for (int i = ndj; i <= nej; i++) {
          if (!yoc[trou[i]]) ndif++;
          if (!yoc[part[i]]) ndif++;
        }
        if (ndif > 2) continue;
      }
      if (ndif == 0) goto L200;
      if (ysaut[j] && j <= kkmax) lesp++;
      ikk_buf[++ijune] = j;
    }
    if (ijune == 0) goto L200;
    for (int j = 1; j <= ijune; j++) stok_buf[j] = hntd(nf, ikk_buf[j]);
    fmul = 0.0;
    nmul = 0;
    if (nespf != 0) {
      ybis = 1;
      fmulbr = 1.0 / (double)(lesp + 1);
      fmul = fmulbr * (double)(nespf + 1) - 1.0;
      nmul = nmul + (int)fmul;
    } else {
      ybis = 0;
    }
    int yet = 0;
    double xam = 0.0;
    int ydeg = 0;
    double hmpi = hmp(nf), hvpi = 0.0;
    if (yen) hvpi = hdig(nf);
    double hmpa = hmp_abs(nf), hvpa = yen ? hdig_abs(nf) : 0.0;
    double eimp = 0, car = 0, eivp = 0, carvp = 0, eib = 0;
    for (int m = 1; m <= metat; m++) {
      double bcalc = 0.0;
      int mncf = (m - 1) * ncf;
      double babs = 0.0;
      for (int j = 1; j <= ijune; j++) bcalc = bcalc + (stok_buf[j] * c[mncf + ikk_buf[j]]);
      for (int j = 1; j <= ijune; j++) babs += fabs(stok_buf[j] * c[mncf + ikk_buf[j]]);
      him[m] = bcalc;
      dmp[m] = emp[m] - hmpi;
      {
        double w = 1.0 + (ybis ? fabs(fmul) : 0.0);
        double kb = bcalc != 0.0 ? U16 * babs / fabs(bcalc) : 0.0;
        double t = fabs(bcalc * bcalc / dmp[m]);
        cond_mp[m] += w * t * (2.0 * kb + U16 * (fabs(emp[m]) + hmpa) / fabs(dmp[m]));
        if (yen) {
          double dv = e[m] - hvpi, dbb = eb[m] - hvpi;
          cond_vp[m] += w * fabs(bcalc * bcalc / dv) * (2.0 * kb + U16 * (fabs(e[m]) + hvpa) / fabs(dv));
          cond_b[m] += w * fabs(bcalc * bcalc / dbb) * (2.0 * kb + U16 * (fabs(eb[m]) + hvpa) / fabs(dbb));
        }
      }
      double cimp = bcalc / dmp[m];
      car = cimp * cimp;
      psimp[m] = psimp[m] + car;
      eimp = bcalc * cimp;
      semp[m] = eimp;
      e2mp[m] = e2mp[m] + eimp;
      comp_add(&ks_mp[m], &kc_mp[m], eimp);
      double xim = fabs(cimp);
      if (ysele) xim = fabs(eimp);
      double deno = dmp[m], eim = eimp;
      if (yen) {
        dvp[m] = e[m] - hvpi;
        double civp = bcalc / (dvp[m]);
        carvp = civp * civp;
        psivp[m] = psivp[m] + carvp;
        eivp = bcalc * civp;
        sevp[m] = eivp;
        e2vp[m] = e2vp[m] + eivp;
        comp_add(&ks_vp[m], &kc_vp[m], eivp);
        xim = fabs(civp);
        if (ysele) xim = fabs(eivp);
        deno = dvp[m];
        eim = eivp;
        db[m] = eb[m] - hvpi;
        double cib = bcalc / (db[m]);
        eib = bcalc * cib;
        e2b[m] = e2b[m] + eib;
        comp_add(&ks_b[m], &kc_b[m], eib);
      }
      if (!(fabs(deno) > 0.05) && !(fabs(eim) < 1.0e-6)) {
        if (ywdeg) ydeg = 1;
      }
      if (xim < teste[m]) {
        if (dpivot < xim) dpivot = xim;
      } else {
        yet = 1;
      }
      if (ymoyen) {
        xim = xim * taum[m];
        vil[m] = xim;
        if (xim > xam) xam = xim;
      }
      venvp[m] = eivp * (fmul + 1.0); /* cipsym/pert1.f:244 */
      if (ybis) {
        e2mp[m] = e2mp[m] + eimp * fmul;
        comp_add(&ks_mp[m], &kc_mp[m], eimp * fmul);
        psimp[m] = psimp[m] + car * fmul;
        if (yen) {
          e2vp[m] = e2vp[m] + eivp * fmul;
          comp_add(&ks_vp[m], &kc_vp[m], eivp * fmul);
          e2b[m] = e2b[m] + eib * fmul;
          comp_add(&ks_b[m], &kc_b[m], eib * fmul);
          psivp[m] = psivp[m] + carvp * fmul;
        }
      }
    }
    (void)yet;
    n_processed++;
    log_candidate(kkmod, nf, xam, him, fmul, nmul);
    {
      double fm = fmul;
      isto(xam, vil, nmul, &fm);
    }
    if (ydeg) xam = 1.0;
    if ((xam > tau) && ymoyen) pie(nec, nts, nps, xam, venvp);
    /* QDPT heff contributions (ybrd) are not restated */
    ietat = ietat + nmul + 1;
  }
L200:
  for (int j = 1; j <= nec; j++) {
    yoc[trou[ndf + j]] = 0;
    yoc[part[ndf + j]] = 0;
  }
  if (nf <= ncf) return;
  if (ne[kk] < nec) return; /* kk >= 1 whenever this is reached from igene */
  {
    int necg = ne[kk], ndk = nd[kk];
    if (yf) return;
    if (ne[nf] > necg) return;
    for (int i = 1; i <= necg; i++) {
      trou[ndf + i] = trou[ndk + i];
      part[ndf + i] = part[ndk + i];
    }
  }
}

/* ------------------------------------------------- cotra (cip/cotra.f) */
static void cotra(int k, int nf) {
  int nt[24], np[24];
  int nup = ne[k];
  int ndf = nd[nf];
  for (int l = 1; l <= nup; l++) {
    nt[l] = trou[ndf + l];
    np[l] = part[ndf + l];
  }
  int jt = 0, jp = 0;
  for (int l = 1; l <= nup; l++) {
    if (nt[l] != 0) trou[ndf + (++jt)] = nt[l];
    if (np[l] != 0) part[ndf + (++jp)] = np[l];
  }
  pert1(k, nf);
}

/* ntps(i,1) == trou(i), ntps(i,2) == part(i) (igene.f:20-21) */
static inline int* ntps(int i, int kr) { return kr == 1 ? &trou[i] : &part[i]; }

/* ------------------------------------------------- igene (cip/igene.f) */
static void igene(int k, int yf, int ym, int yd) {
  int nf = ncf + 1;
  int ndk = nd[k], ndf = nd[nf];
  int nec = ne[k];
  if (nec != 0)
    for (int ir = 1; ir <= nec; ir++) {
      trou[ndf + ir] = trou[ndk + ir];
      part[ndf + ir] = part[ndk + ir];
    }
  if (nec == 0 && ym) return;
  if (nec == 1 && yd) return;
  /* monoexcitations (igene.f:36-84) */
  int nec1 = nec + 1;
  ne[nf] = nec + 1;
  for (int ks = 1; ks <= 2; ks++) {
    int igel = igels_[ks], n = norbs_[ks], nbor = noc_[ks], nbor1 = nbor + 1;
    for (int ii = igel; ii <= nbor; ii++) {
      trou[ndf + nec1] = ii;
      int iis = itsym[ii];
      for (int jj = nbor1; jj <= n; jj++) {
        if (YOCD(ii, k) || YOCD(jj, k)) continue;
        part[ndf + nec1] = jj;
        int jjs = itsym[jj];
        int ijs = its[iis][jjs];
        if (ijs == 1) pert1(k, nf);
        if (nec == 0) continue;
        for (int kr = 1; kr <= 2; kr++) {
          for (int lk = 1; lk <= nec; lk++) {
            int la = *ntps(ndk + lk, kr);
            int ls = ispin[la] + 1;
            int las = itsym[la];
            int na1, na2;
            if (kr <= 1) {
              na1 = igels_[ls];
              if (ls == ks) na1 = ii + 1;
              na2 = noc_[ls];
            } else {
              na1 = noc_[ls] + 1;
              if (ls == ks) na1 = jj + 1;
              na2 = norbs_[ls];
            }
            if (na1 > na2) continue;
            for (int ll = na1; ll <= na2; ll++) {
              if (ll == la || ll == ii || ll == jj) continue;
              *ntps(ndf + lk, kr) = ll;
              int lls = itsym[ll];
              int kls = its[las][lls];
              int ijkls = its[ijs][kls];
              if (ijkls == 1) pert1(k, nf);
              *ntps(ndf + lk, kr) = la;
            }
          }
        }
      }
    }
  }
  if (nec < 1) return;
  if (ym && nec == 1 && !yion) return;
  if (nec == 2 && yd) return;
  /* same excitation degree (igene.f:91-145) */
  ne[nf] = nec;
  for (int lk = 1; lk <= nec; lk++) {
    int lk1 = lk + 1;
    for (int kr = 1; kr <= 2; kr++) {
      int la = *ntps(ndk + lk, kr);
      int ls = ispin[la] + 1;
      int las = itsym[la];
      int na1, na2;
      if (kr <= 1) {
        na1 = igels_[ls];
        na2 = noc_[ls];
      } else {
        na1 = noc_[ls] + 1;
        na2 = norbs_[ls];
      }
      for (int ll = na1; ll <= na2; ll++) {
        int ll1 = ll + 1;
        if (ll == la) continue;
        *ntps(ndf + lk, kr) = ll;
        int lls = itsym[ll];
        int lalls = its[las][lls];
        if (lalls == 1) pert1(k, nf);
        if (lk == nec) continue;
        for (int lkp = lk1; lkp <= nec; lkp++) {
          int lb = *ntps(ndk + lkp, kr);
          int lbs = ispin[lb] + 1;
          if (lbs == ls && ll >= na2) continue; /* go to 568: no restore */
          int lbsy = itsym[lb];
          int nb1, nb2;
          if (kr == 2) {
            nb2 = norbs_[lbs];
            nb1 = noc_[lbs] + 1;
          } else {
            nb2 = noc_[lbs];
            nb1 = igels_[lbs];
          }
          if (ll != lb) {
            if (ls == lbs) nb1 = ll1;
            for (int ii = nb1; ii <= nb2; ii++) {
              if (ii == lb) continue;
              if (ii == la) continue;
              *ntps(ndf + lkp, kr) = ii;
              *ntps(ndf + lk, kr) = ll;
              int iis = itsym[ii];
              int ibs = its[lbsy][iis];
              if (its[ibs][lalls] == 1) pert1(k, nf);
            }
          }
          *ntps(ndf + lkp, kr) = lb;
        }
      }
      *ntps(ndf + lk, kr) = la;
    }
  }
  /* hole-particle pair replacement (igene.f:146-198) */
  for (int lk = 1; lk <= nec; lk++) {
    int la = trou[ndk + lk];
    int ls = ispin[la] + 1;
    int las = itsym[la];
    int na1 = igels_[ls], na2 = noc_[ls];
    for (int lkp = 1; lkp <= nec; lkp++) {
      int lb = part[ndk + lkp];
      int lbs = ispin[lb] + 1;
      int nb1 = noc_[lbs] + 1, nb2 = norbs_[lbs];
      int lbsy = itsym[lb];
      int lalbs = its[las][lbsy];
      int ntsp = ls - lbs;
      for (int ll = na1; ll <= na2; ll++) {
        if (ll == la) continue;
        int lls = itsym[ll];
        for (int ii = nb1; ii <= nb2; ii++) {
          if (ii == lb) continue;
          part[ndf + lkp] = ii;
          trou[ndf + lk] = ll;
          int iis = itsym[ii];
          int lis = its[lls][iis];
          int liabs = its[lis][lalbs];
          if (liabs == 1) pert1(k, nf);
        }
      }
      if (ntsp == 0) {
        int lsp = -ls + 3; /* spin change */
        int nocu = noc_[lsp], nocu1 = nocu + 1, igelu = igels_[lsp], norbu = norbs_[lsp];
        for (int ll = igelu; ll <= nocu; ll++) {
          int lls = itsym[ll];
          for (int ii = nocu1; ii <= norbu; ii++) {
            trou[ndf + lk] = ll;
            part[ndf + lkp] = ii;
            int iis = itsym[ii];
            int lis = its[lls][iis];
            int liabs = its[lis][lalbs];
            if (liabs == 1) pert1(k, nf);
          }
        }
      }
      part[ndf + lkp] = lb; /* 588: terminal statement of the lkp loop */
    }
    trou[ndf + lk] = la;
  }
  if (nec == 3 && yd) return;
  if (nec == 2 && ym) return;
  /* one de-excitation (igene.f:201-290) */
  ne[nf] = nec - 1;
  for (int lk = 1; lk <= nec; lk++) {
    int la = trou[ndk + lk];
    int ls = ispin[la] + 1;
    int las = itsym[la];
    for (int lkp = 1; lkp <= nec; lkp++) {
      int lb = part[ndk + lkp];
      int lbs = ispin[lb] + 1;
      if (ls != lbs) {
        part[ndf + lkp] = lb;
        continue;
      }
      int lbsy = itsym[lb];
      trou[ndf + lk] = 0;
      part[ndf + lkp] = 0;
      int lalbs = its[las][lbsy];
      if (lalbs == 1) cotra(k, nf);
      for (int lkt = 1; lkt <= nec; lkt++) {
        int lat = trou[ndk + lkt];
        int lts = ispin[lat] + 1;
        int lbt = part[ndk + lkt];
        /* change of a hole */
        if (lkt != lk) {
          int kr = 1;
          int ici = itsym[lat];
          int na1 = igels_[lts], na2 = noc_[lts];
          int nevi2 = lat;
          int doit = 1, nevi1 = 0;
          if (ls != lts) {
            nevi1 = 0;
          } else {
            if (lkt - lk <= 0)
              doit = 0;
            else
              nevi1 = la;
          }
          if (doit) {
            for (int ii = na1; ii <= na2; ii++) {
              if (ii == nevi1 || ii == nevi2) continue;
              *ntps(ndf + lkt, kr) = ii;
              trou[ndf + lk] = 0;
              part[ndf + lkp] = 0;
              int iici = its[ici][itsym[ii]];
              if (its[iici][lalbs] == 1) cotra(k, nf);
            }
            *ntps(ndf + lkt, kr) = *ntps(ndk + lkt, kr);
          }
        }
        /* change of a particle (label 624) */
        {
          int lps = ispin[lbt] + 1;
          int kr = 2;
          int ici = itsym[lbt];
          int na1 = noc_[lps] + 1, na2 = norbs_[lps];
          int nevi2 = lbt;
          if (lkt == lkp) continue;
          int nevi1;
          if (ls != lps) {
            nevi1 = 0;
          } else {
            if (lkt - lkp <= 0) continue;
            nevi1 = lb;
          }
          for (int ii = na1; ii <= na2; ii++) {
            if (ii == nevi1 || ii == nevi2) continue;
            *ntps(ndf + lkt, kr) = ii;
            trou[ndf + lk] = 0;
            part[ndf + lkp] = 0;
            int iici = its[ici][itsym[ii]];
            if (its[iici][lalbs] == 1) cotra(k, nf);
          }
          *ntps(ndf + lkt, kr) = *ntps(ndk + lkt, kr);
        }
      }
      part[ndf + lkp] = lb;
    }
    trou[ndf + lk] = la;
  }
  /* two de-excitations (igene.f:291-350) */
  if (nec == 2 && (yd || yf)) return;
  if (nec == 3 && ym) return;
  if (nec == 4 && yd) return;
  int necm = nec - 1;
  ne[nf] = nec - 2;
  for (int lt1 = 1; lt1 <= necm; lt1++) {
    int lt1p = lt1 + 1;
    int lat = trou[ndk + lt1];
    int lats = ispin[lat] + 1;
    int ilat = itsym[lat];
    for (int lt2 = lt1p; lt2 <= nec; lt2++) {
      int lbt = trou[ndk + lt2];
      int lbts = ispin[lbt] + 1;
      int nts_ = lats - lbts;
      int ilbt = itsym[lbt];
      int ilab = its[ilat][ilbt];
      for (int lp1 = 1; lp1 <= necm; lp1++) {
        int lp1p = lp1 + 1;
        int lcp = part[ndk + lp1];
        int lcps = ispin[lcp] + 1;
        int ilcp = itsym[lcp];
        for (int lp2 = lp1p; lp2 <= nec; lp2++) {
          int ldp = part[ndk + lp2];
          int ldps = ispin[ldp] + 1;
          int go = 0;
          if (nts_ != 0) {
            if (lcps != ldps) go = 1;
          } else {
            if (lcps == lats && ldps == lats) go = 1;
          }
          if (go) {
            trou[ndf + lt1] = 0;
            trou[ndf + lt2] = 0;
            part[ndf + lp1] = 0;
            part[ndf + lp2] = 0;
            int ildp = itsym[ldp];
            int ilcd = its[ilcp][ildp];
            int ilabcd = its[ilab][ilcd];
            if (ilabcd == 1) cotra(k, nf);
          }
          part[ndf + lp2] = ldp;
        }
        part[ndf + lp1] = lcp;
      }
      trou[ndf + lt2] = lbt;
    }
    trou[ndf + lt1] = lat;
  }
}

/* ------------------------------------------------- pertu (cip/pertu.f) */
static void pertu(void) {
  int nsy = isym;
  int nf = ncf + 1;
  int yd = 0, ym = 0, yf = 0;
  for (int k = 1; k <= ncf; k++) {
    if (ne[k] == 1) ym = 1;
    if (ne[k] == 0) yd = 1;
    if (ne[k] == 2) yf = 1;
  }
  if (ym) yf = ym;
  cur_src = 0;
  if (!yion && yf) {
    if (!(yd || isz != 0)) {
      if (nsy == 1) {
        ne[nf] = 0;
        if (run_pertu_ref) pert1(0, nf);
      }
    }
    ne[nf] = 1;
    if (ym) {
      int ndf = nd[nf] + 1;
      if (isz != 0) {
        int igel = igela, n = mnorb, ip1 = nocb + 1, itm = noca;
        for (int it = igel; it <= itm; it++) {
          int ist = itsym[it];
          for (int ip = ip1; ip <= n; ip++) {
            if (its[ist][itsym[ip]] != nsy) continue;
            part[ndf] = ip;
            trou[ndf] = it;
            if (run_pertu_ref) pert1(0, nf);
          }
        }
      } else {
        for (int is = 1; is <= 2; is++) {
          int igel = igels_[is], itm = noc_[is], ip1 = itm + 1, n = norbs_[is];
          for (int it = igel; it <= itm; it++) {
            int ist = itsym[it];
            for (int ip = ip1; ip <= n; ip++) {
              if (its[ist][itsym[ip]] != nsy) continue;
              part[ndf] = ip;
              trou[ndf] = it;
              if (run_pertu_ref) pert1(0, nf);
            }
          }
        }
      }
    }
  }
  cur_src = 1;
  for (int k = 1; k <= ncf; k++) {
    if (!ygen[k]) continue;
    if (ysaut[k]) continue;
    if (gen_mask && !gen_mask[k]) continue;
    igene(k, yf, ym, yd);
  }
}

/* --------------------------------------------- diexcit (cip/diexcit.f) */
static int* irapid;

static void diexcit_one(int ii, int jj, int kk, int ll, int nspin, int yijkl, double* hijkl_p) {
  if (samp_M > 1 && (samp_seq++ % samp_M) != samp_m) return;
  /* isp(4,3) data 0,1,0,1, 0,0,0,0, 0,1,1,0 (column-major isp(i,isa)) */
  static const int ISP[4][5] = {{0}, {0, 0, 1, 0, 1}, {0, 0, 0, 0, 0}, {0, 0, 1, 1, 0}};
  int nf = ncf + 1, ndf = nd[nf];
  int ysyspi = !yijkl;
  double haj = ai(ii, kk, jj, ll), hak = 0.0;
  if (nspin > 1) hak = ai(ii, ll, jj, kk);
  for (int isa = 1; isa <= nspin; isa++) {
    int iso = ii + ISP[isa][1] * norb;
    int jso = jj + ISP[isa][2] * norb;
    int kso = kk + ISP[isa][3] * norb;
    int lso = ll + ISP[isa][4] * norb;
    int yspi = 0;
    if (!yorper[iorb[iso]] || !yorper[iorb[jso]] || !yorper[iorb[kso]] || !yorper[iorb[lso]])
      goto L1005; /* note: hijkl keeps its previous value (diexcit.f:188-194) */
    *hijkl_p = 0.0;
    if (isa <= 2) *hijkl_p = haj;
    if (isa >= 2) *hijkl_p = *hijkl_p - hak;
    yspi = 0;
  L1800:;
    {
      double hijkl = *hijkl_p;
      yoc[iso] = 1;
      yoc[jso] = 1;
      yoc[kso] = 1;
      yoc[lso] = 1;
      int ndf1 = ndf + 1, ndf2 = ndf + 2;
      part[ndf1] = kso;
      part[ndf2] = lso;
      trou[ndf2] = jso;
      trou[ndf1] = iso;
      for (int k = 1; k <= ncf; k++) {
        int i = 0;
        if (YOCD(iso, k)) i++;
        if (YOCD(jso, k)) i++;
        if (YOCD(kso, k)) i++;
        if (YOCD(lso, k)) i++;
        irapid[k] = i;
      }
      int yquick = !(yocs[iso] || yocs[jso] || yocs[kso] || yocs[lso]);
      if (yquick && hijkl == 0.0) goto L2000;
      for (int kkk = 1; kkk <= ncf; kkk++) {
        if (!ygen[kkk]) continue;
        int nec = ne[kkk];
        int yf = (nec == 0);
        if (ysaut[kkk]) continue;
        if (gen_mask && !gen_mask[kkk]) continue;
        int nespf = nesp[kkk];
        int ybis = nespf > 0;
        if (yspi && !yef1[kkk]) continue;
        int kkkmax = kkk + nespf;
        int lesp = 0;
        int ndk = nd[kkk];
        int nec2 = nec + 2;
        ne[nf] = nec2;
        int ijune = 1;
        ikk_buf[1] = kkk;
        stok_buf[1] = hijkl;
        if (!yquick) {
          if (nec != 0) {
            if (YOCD(iso, kkk) || YOCD(jso, kkk) || YOCD(kso, kkk) || YOCD(lso, kkk)) continue;
          }
          /* owner test (diexcit.f:246-259) */
          int owned = 0;
          for (int j = 1; j < kkk; j++) {
            if (!ygen[j]) continue;
            if (irapid[j] == 0) continue;
            int ndif = ne[j] - nec + 2 - irapid[j];
            if (ndif >= 2) continue;
            if (yf) { owned = 1; break; }
            for (int l = 1; l <= nec; l++) {
              if (!YOCD(trou[ndk + l], j)) ndif++;
              if (!YOCD(part[ndk + l], j)) ndif++;
            }
            if (ndif > 2) continue;
            owned = 1;
            break;
          }
          if (owned) continue;
        }
        /* L310 */
        if (!yf)
          for (int i = 1; i <= nec; i++) {
            part[ndf2 + i] = part[ndk + i];
            trou[ndf2 + i] = trou[ndk + i];
          }
        int drop = 0;
        if (!yquick) {
          for (int j = kkk + 1; j <= ncf; j++) {
            if (irapid[j] == 0) continue;
            int ndif = ne[j] - nec + 2 - irapid[j];
            if (ndif > 2) continue;
            if (!yf) {
              for (int l = 1; l <= nec; l++) {
                if (!YOCD(trou[ndk + l], j)) ndif++;
                if (!YOCD(part[ndk + l], j)) ndif++;
              }
              if (ndif > 2) continue;
            }
            if (ndif == 0) { drop = 1; break; }
            if (j <= kkkmax) lesp++;
            ikk_buf[++ijune] = j;
          }
        }
        if (drop) continue; /* go to 900 */
        {
          int i = 0;
          for (int m = 1; m <= ijune; m++) {
            int j = ikk_buf[m];
            double bcalc = (m == 1) ? stok_buf[1] : hntd(nf, j);
            if (bcalc == 0.0) continue;
            i++;
            stok_buf[i] = bcalc;
            ikk_buf[i] = j;
          }
          ijune = i;
        }
        if (ijune == 0) continue;
        int yefsk = yef1[kkk];
        int ysbrd = yefsk || ysyspi;
        if (ysbrd) {
          ybis = 1;
          if (!yefsk) nespf = nespf + nespf + 1;
        }
        double fmulbr = 1.0 / (double)(lesp + 1);
        double fmul = fmulbr * (double)(nespf + 1) - 1.0;
        int nmul = (int)fmul;
        double vil[64] = {0}, him[64], venvp[64];
        double xam = 0.0;
        int ydeg = 0;
        double hmpi = hmp(nf), hvpi = 0.0;
        if (yen) hvpi = hdig(nf);
        double hmpa = hmp_abs(nf), hvpa = yen ? hdig_abs(nf) : 0.0;
        for (int m = 1; m <= metat; m++) {
          double bcalc = 0.0, babs = 0.0;
          int mncf = (m - 1) * ncf;
          for (int j = 1; j <= ijune; j++) bcalc = bcalc + (stok_buf[j] * c[mncf + ikk_buf[j]]);
          for (int j = 1; j <= ijune; j++) babs += fabs(stok_buf[j] * c[mncf + ikk_buf[j]]);
          him[m] = bcalc;
          double dmpm = emp[m] - hmpi;
          {
            double w = 1.0 + (ybis ? fabs(fmul) : 0.0);
            double kb = bcalc != 0.0 ? U16 * babs / fabs(bcalc) : 0.0;
            cond_mp[m] += w * fabs(bcalc * bcalc / dmpm) * (2.0 * kb + U16 * (fabs(emp[m]) + hmpa) / fabs(dmpm));
            if (yen) {
              double dv = e[m] - hvpi, dbb = eb[m] - hvpi;
              cond_vp[m] += w * fabs(bcalc * bcalc / dv) * (2.0 * kb + U16 * (fabs(e[m]) + hvpa) / fabs(dv));
              cond_b[m] += w * fabs(bcalc * bcalc / dbb) * (2.0 * kb + U16 * (fabs(eb[m]) + hvpa) / fabs(dbb));
            }
          }
          double cimp = bcalc / dmpm;
          double car = cimp * cimp;
          psimp[m] = psimp[m] + car;
          double eimp = bcalc * cimp;
          semp[m] = eimp;
          e2mp[m] = e2mp[m] + eimp;
          comp_add(&ks_mp[m], &kc_mp[m], eimp);
          double xim = fabs(cimp);
          if (ysele) xim = fabs(eimp);
          double deno = dmpm, eim = eimp;
          double eivp = 0, carvp = 0, eib = 0;
          if (yen) {
            double dvpm = e[m] - hvpi;
            double civp = bcalc / dvpm;
            carvp = civp * civp;
            psivp[m] = psivp[m] + carvp;
            eivp = bcalc * civp;
            sevp[m] = eivp;
            e2vp[m] = e2vp[m] + eivp;
            comp_add(&ks_vp[m], &kc_vp[m], eivp);
            xim = fabs(civp);
            if (ysele) xim = fabs(eivp);
            deno = dvpm;
            eim = eivp;
            double dbm = eb[m] - hvpi;
            double cib = bcalc / dbm;
            eib = bcalc * cib;
            e2b[m] = e2b[m] + eib;
            comp_add(&ks_b[m], &kc_b[m], eib);
          }
          if (!(fabs(deno) > 0.05) && !(fabs(eim) < 1.0e-6)) {
            if (ywdeg) ydeg = 1;
          }
          if (xim < teste[m]) {
            if (dpivot < xim) dpivot = xim;
          }
          if (ymoyen) {
            xim = xim * taum[m];
            vil[m] = xim;
            if (xim > xam) xam = xim;
          }
          venvp[m] = eivp * (fmul + 1.0); /* cipsym/diexcit.f:446 */
          if (ybis) {
            e2mp[m] = e2mp[m] + eimp * fmul;
            comp_add(&ks_mp[m], &kc_mp[m], eimp * fmul);
            psimp[m] = psimp[m] + car * fmul;
            if (yen) {
              e2vp[m] = e2vp[m] + eivp * fmul;
              comp_add(&ks_vp[m], &kc_vp[m], eivp * fmul);
              e2b[m] = e2b[m] + eib * fmul;
              comp_add(&ks_b[m], &kc_b[m], eib * fmul);
              psivp[m] = psivp[m] + carvp * fmul;
            }
          }
        }
        ietat = ietat + nmul + 1;
        n_processed++;
        log_candidate(kkk, nf, xam, him, fmul, nmul);
        if (ymoyen) {
          double fm = fmul;
          isto(xam, vil, nmul, &fm);
          int nex = ne[nf];
          int nts[16], nps[16];
          for (int i = 1; i <= nex; i++) {
            nts[i] = trou[ndf + i];
            nps[i] = part[ndf + i];
          }
          if (ydeg) xam = 1.0;
          if (xam > tau) pie(nex, nts, nps, xam, venvp);
        }
      }
    }
  L1005:
    yoc[iso] = 0;
    yoc[jso] = 0;
    yoc[kso] = 0;
    yoc[lso] = 0;
    if (!ysyspi) goto L2000;
    if (yspi) goto L2000;
    yspi = 1;
    iso = isytr1[iso];
    jso = isytr1[jso];
    kso = isytr1[kso];
    lso = isytr1[lso];
    goto L1800;
  L2000:;
  }
}

static void diexcit(void) {
  double hijkl = 0.0; /* persists across calls, as the Fortran local does */
  int igel = igela, nbor = noc2, nbor1 = noc1 + 1, n = norb, nm1 = n - 1;
  int nbi = nbor - 1;
  cur_src = 2;
  /* iva = 1 : ii = jj, kk = ll */
  for (int ii = igel; ii <= nbor; ii++) {
    int iis = itsym[ii];
    if (its[iis][iis] != 1) continue;
    for (int kk = nbor1; kk <= n; kk++) {
      int kks = itsym[kk];
      if (its[kks][kks] != 1) continue;
      diexcit_one(ii, ii, kk, kk, 1, 1, &hijkl);
    }
  }
  /* iva = 2 : ii = jj, kk < ll */
  if (nm1 != nbor) {
    for (int ii = igel; ii <= nbor; ii++) {
      int iis = itsym[ii];
      if (its[iis][iis] != 1) continue;
      for (int kk = nbor1; kk <= nm1; kk++) {
        int kks = itsym[kk];
        for (int ll = kk + 1; ll <= n; ll++) {
          if (its[kks][itsym[ll]] == 1) diexcit_one(ii, ii, kk, ll, 1, 0, &hijkl);
        }
      }
    }
  }
  if (nbi <= 0) return;
  /* iva = 3 : ii < jj, kk = ll */
  for (int ii = igel; ii <= nbi; ii++) {
    int iis = itsym[ii];
    for (int jj = ii + 1; jj <= nbor; jj++) {
      if (its[iis][itsym[jj]] != 1) continue;
      for (int kk = nbor1; kk <= n; kk++) {
        int kks = itsym[kk];
        if (its[kks][kks] != 1) continue;
        diexcit_one(ii, jj, kk, kk, 1, 0, &hijkl);
      }
    }
  }
  /* iva = 4 : ii < jj, kk < ll */
  if (nm1 == nbor) return;
  for (int ii = igel; ii <= nbi; ii++) {
    int iis = itsym[ii];
    for (int jj = ii + 1; jj <= nbor; jj++) {
      int ijs = its[iis][itsym[jj]];
      for (int kk = nbor1; kk <= nm1; kk++) {
        int kks = itsym[kk];
        for (int ll = kk + 1; ll <= n; ll++) {
          int kls = its[kks][itsym[ll]];
          if (its[ijs][kls] == 1) diexcit_one(ii, jj, kk, ll, 3, 0, &hijkl);
        }
      }
    }
  }
}

/* ---------------------------------------------- S construction (deter) */
static int* kex_lists[10]; /* per excitation degree: holes then particles */
static int kex_cnt[10];    /* number of determinants per degree */
static int kex_cap[10];
static int kf_ref = 0;
static int g_ncf_cap = 0;

static void kex_push(int nec, const int* itab) {
  if (kex_cnt[nec] >= kex_cap[nec]) {
    kex_cap[nec] = kex_cap[nec] * 2 + 64;
    kex_lists[nec] = (int*)realloc(kex_lists[nec], sizeof(int) * (size_t)kex_cap[nec] * 2 * nec);
  }
  memcpy(kex_lists[nec] + (size_t)kex_cnt[nec] * 2 * nec, itab, sizeof(int) * 2 * (size_t)nec);
  kex_cnt[nec]++;
}

/* lec60.f: read the determinants of unit 60 with v >= tdet */
static void lec60(FILE* f) {
  rec_t r = {0};
  int ndet = 0;
  rewind(f);
  while (rec_read(f, &r)) {
    int mw = rec_i4(&r), nw = rec_i4(&r);
    int* idet = (int*)xcalloc((size_t)mw + 1, sizeof(int));
    int* necst = (int*)xcalloc((size_t)nw + 1, sizeof(int));
    double* v = (double*)xcalloc((size_t)nw + 1, sizeof(double));
    for (int i = 1; i <= mw; i++) idet[i] = rec_i4(&r);
    for (int i = 1; i <= nw; i++) necst[i] = rec_i4(&r);
    for (int i = 1; i <= nw; i++) v[i] = rec_r8(&r);
    int myy = 0;
    for (int l = 1; l <= nw; l++) {
      int nec = necst[l];
      if (nec > 8) die("degre d excitation %d depasse les possibilites du programme", nec);
      if (v[l] < tdet) {
        myy += 2 * nec;
        continue;
      }
      ndet++;
      if (ndet > maxdet) {
        if (lecdet == 3) goto done;
        die("trop de determinants selectionnes sur la file60");
      }
      int itab[20];
      for (int s = 1; s <= nec; s++) {
        itab[s - 1] = idet[++myy];
        itab[s - 1 + nec] = idet[++myy];
      }
      if (nec == 0) {
        if (isz != 0) continue;
        kf_ref++;
        if (kf_ref != 1) {
          kf_ref--;
          printf(" fondamental deja present\n");
        }
        continue;
      }
      kex_push(nec, itab);
    }
    free(idet);
    free(necst);
    free(v);
  }
done:
  free(r.b);
  rewind(f);
}

/* cas.f:64-110: the increasing n-tuples of 1..noac in lexicographic order
   (istr starts at (1, .., n-1, n-1) so that the first step gives 1..n).
   Returns their number; the tuples go to out[ii*10 + k], k = 0..n-1. */
#define NIIZ 25000
static int cas_strings(int n, int noac, int* out) {
  int istr[16] = {0};
  for (int k = 1; k <= n; k++) istr[k] = k;
  if (n != 0) istr[n] = n - 1;
  int ii = 0, i = n + 1;
L10:
  i = i - 1;
  if (i == 0) return ii;
L14:;
  int newoc = istr[i] + 1;
  if (newoc > (noac - n + i)) goto L10;
  istr[i] = newoc;
  for (int k = i + 1; k <= n; k++) istr[k] = istr[k - 1] + 1;
  i = n;
  ii = ii + 1;
  if (ii > NIIZ) die("  trop de combinaisons: max=%d", NIIZ);
  for (int k = 1; k <= n; k++) out[(size_t)(ii - 1) * 10 + (k - 1)] = istr[k];
  goto L14;
}

/* cas.f:111-166: one string's holes (orbitals numac(1..noc) it leaves
   empty) then particles (numac(noc+1..noac) it fills), as orbital numbers.
   Returns the hole count; *np gets the particle count. */
static int cas_excitation(const int* occ, int n, int noc, int* mtp, int* np) {
  unsigned char yocc[520] = {0};
  for (int k = 1; k <= n; k++) yocc[occ[k - 1]] = 1;
  int itp = 0;
  for (int k = 1; k <= noc; k++)
    if (!yocc[k]) {
      if (itp >= 10) die("more than 10 holes and particles in one string of the CAS");
      mtp[++itp] = numac[k];
    }
  int nt = itp;
  for (int k = noc + 1; k <= noac; k++)
    if (yocc[k]) {
      if (itp >= 10) die("more than 10 holes and particles in one string of the CAS");
      mtp[++itp] = numac[k];
    }
  *np = itp - nt;
  return nt;
}

/* cas.f: the CAS determinants of symmetry nusym with at most nemax
   excitations, alpha strings outer and beta strings inner, into the
   per-degree lists that deter.f:478-567 turns into S (yion is rejected
   before, so nalfa = nbeta = noc = (nelac+1)/2) */
static void cas(void) {
  int nalfa = (nelac + 1) / 2, nbeta = nalfa;
  if (nelac > 20) die(" trop d electrons actifs  maximum 20");
  int noc = nalfa;
  if (nalfa > noac) die("more active electrons of one spin (%d) than active orbitals (%d)", nalfa, noac);
  for (int k = 1; k <= noac; k++)
    if (numac[k] < 1 || numac[k] > norb) die("numac(%d)=%d is not an orbital", k, numac[k]);
  int* noma = (int*)xcalloc((size_t)NIIZ * 10 + 10, sizeof(int));
  int* nomb = (int*)xcalloc((size_t)NIIZ * 10 + 10, sizeof(int));
  int nca = cas_strings(nalfa, noac, noma);
  int ncb = cas_strings(nbeta, noac, nomb);
  int *nta = (int*)xcalloc((size_t)NIIZ + 2, sizeof(int)), *npa = (int*)xcalloc((size_t)NIIZ + 2, sizeof(int));
  int *ntb = (int*)xcalloc((size_t)NIIZ + 2, sizeof(int)), *npb = (int*)xcalloc((size_t)NIIZ + 2, sizeof(int));
  int mtp[12];
  for (int ia = 1; ia <= (nca > 1 ? nca : 1); ia++) {
    int* row = noma + (size_t)(ia - 1) * 10;
    nta[ia] = cas_excitation(row, nca ? nalfa : 0, noc, mtp, &npa[ia]);
    for (int k = 1; k <= nta[ia] + npa[ia]; k++) row[k - 1] = mtp[k];
  }
  for (int ib = 1; ib <= ncb; ib++) {
    int* row = nomb + (size_t)(ib - 1) * 10;
    ntb[ib] = cas_excitation(row, nbeta, noc, mtp, &npb[ib]);
    for (int k = 1; k <= ntb[ib] + npb[ib]; k++) row[k - 1] = mtp[k];
  }
  int ndet = 0;
  for (int ia = 1; ia <= (nca > 1 ? nca : 1); ia++) {
    int kta = nta[ia], kpa = npa[ia];
    int nts[24], nps[24];
    const int* ra = noma + (size_t)(ia - 1) * 10;
    for (int k = 1; k <= kta; k++) nts[k] = ra[k - 1];
    for (int k = 1; k <= kpa; k++) nps[k] = ra[k - 1 + kta];
    for (int ib = 1; ib <= ncb; ib++) {
      int ktb = ntb[ib], kpb = npb[ib];
      const int* rb = nomb + (size_t)(ib - 1) * 10;
      for (int k = 1; k <= ktb; k++) nts[k + kta] = rb[k - 1] + norb;
      for (int k = 1; k <= kpb; k++) nps[k + kpa] = rb[k - 1 + ktb] + norb;
      int nect = kta + ktb, necp = kpa + kpb;
      if (nect != necp) die("  attention necp et nect sont differents %d %d", nect, necp);
      int nec = necp;
      if (g_sym_variant && nec > nemax) continue; /* cip/cas.f has no nemax */
      int is = 1;
      for (int i = 1; i <= nec; i++) {
        int jps = itsym[nps[i]];
        is = its[is][itsym[nts[i]]];
        is = its[is][jps];
      }
      if (nusym == 0) nusym = is;
      if (is != nusym) continue;
      ndet = ndet + 1;
      if (ndet > UNIT4_NDETZ) die(" espace actif trop grand  maximum=%d", UNIT4_NDETZ);
      if (nec == 0) {
        if (isz != 0) continue;
        kf_ref++;
        if (kf_ref != 1) {
          kf_ref--;
          printf(" fondamental deja present\n");
        }
        continue;
      }
      if (nec > 8) die("CAS determinant of excitation degree %d above 8", nec);
      int itab[20];
      for (int s = 1; s <= nec; s++) {
        itab[s - 1] = nts[s];
        itab[s - 1 + nec] = nps[s];
      }
      kex_push(nec, itab);
    }
  }
  printf("   determinants engendres %d\n", ndet);
  free(noma); free(nomb); free(nta); free(npa); free(ntb); free(npb);
}

/* shell.f: Shell's diminishing-increment sort of a[1..n] into decreasing
   order, carrying ind along; log2(n) passes with increments n/2, n/4, ..
   (the pass count from single-precision logarithms, as shell.f computes it) */
static void shell(double* a, int* ind, int n) {
  const double aln2i = (double)(1.0f / 0.69314748f), tiny = (double)1.0e-5f;
  int lognb2 = (int)((double)logf((float)n) * aln2i + tiny);
  int m = n;
  for (int nn = 1; nn <= lognb2; nn++) {
    m = m / 2;
    int k = n - m;
    for (int j = 1; j <= k; j++) {
      int i = j;
      for (;;) {
        int l = i + m;
        if (!(a[l] > a[i])) break;
        double t = a[i];
        a[i] = a[l];
        a[l] = t;
        int indi = ind[i];
        ind[i] = ind[l];
        ind[l] = indi;
        i = i - m;
        if (i < 1) break;
      }
    }
  }
}

/* transf.f: validate, sort and append one determinant (nt/np 1-based) */
static int tr_nt[12], tr_np[12];
static int g_ntp_used = 0;
static void transf(int nec) {
  if (nec == 0) {
    ncf++;
    ne[ncf] = 0;
    nd[ncf] = 0;
    trou[1] = 0;
    part[1] = 0;
    if (isz != 0) ncf--;
    isym = 1;
    if (g_ntp_used < 1) g_ntp_used = 1;
    return;
  }
  if (nec > 1) {
    for (int i = 1; i <= nec - 1; i++)
      for (int j = i + 1; j <= nec; j++) {
        if (!(tr_nt[j] > tr_nt[i])) { int n = tr_nt[j]; tr_nt[j] = tr_nt[i]; tr_nt[i] = n; }
        if (!(tr_np[j] > tr_np[i])) { int n = tr_np[j]; tr_np[j] = tr_np[i]; tr_np[i] = n; }
      }
  }
  int is = 1, ls = 0;
  if (tr_nt[1] < igela) die("1 spin orbitale est hors de l espace de base");
  if (tr_np[nec] > mnorb && !yion) die("1 spin orbitale est hors de l espace de base");
  if (tr_nt[nec] > nocb) die("1 spin orbitale est hors de l espace de base");
  if (tr_np[nec] <= noca) die("1 spin orbitale est hors de l espace de base");
  for (int i = 1; i <= nec; i++) {
    if (!(tr_nt[i] <= noca) && tr_nt[i] < igelb) die("1 spin orbitale est hors de l espace de base");
    if (!(tr_np[i] > nocb)) {
      if (tr_np[i] > norb) {
        if (yion) return;
        die("1 spin orbitale est hors de l espace de base");
      }
      if (tr_np[i] <= noca) die("1 spin orbitale est hors de l espace de base");
    }
    is = its[is][itsym[tr_nt[i]]];
    is = its[is][itsym[tr_np[i]]];
    ls = ls + ispin[tr_np[i]];
    ls = ls - ispin[tr_nt[i]];
  }
  if (isym == 0) isym = is;
  if (!yion && is != isym) die("determinant de mauvaise symetrie");
  if (ls != isz) die("mauvais spin");
  int ndk;
  if (ncf == 0) {
    ndk = 0;
  } else {
    for (int i = 1; i <= ncf; i++) {
      if (ne[i] != nec) continue;
      int d = nd[i], same = 1;
      for (int j = 1; j <= nec; j++)
        if (trou[d + j] != tr_nt[j] || part[d + j] != tr_np[j]) { same = 0; break; }
      if (same) return;
    }
    ndk = nd[ncf] + ne[ncf];
    if (ne[ncf] == 0) ndk = nd[ncf] + 1;
  }
  ncf++;
  if (ncf > g_ncf_cap) die("trop de determinants dans s");
  for (int j = 1; j <= mnorb; j++) YOCD(j, ncf) = 0;
  ne[ncf] = nec;
  nd[ncf] = ndk;
  for (int j = 1; j <= nec; j++) {
    yocs[tr_nt[j]] = 1;
    yocs[tr_np[j]] = 1;
    YOCD(tr_nt[j], ncf) = 1;
    YOCD(tr_np[j], ncf) = 1;
    trou[ndk + j] = tr_nt[j];
    part[ndk + j] = tr_np[j];
  }
  if (ndk + nec > g_ntp_used) g_ntp_used = ndk + nec;
}

/* deter.f:478-567 for ntrsy == 1 (no spatial degeneracy operations) */
static void build_space(void) {
  ncf = 0;
  if (kf_ref) transf(0);
  for (int nec = 1; nec <= 8; nec++) {
    for (int d = 0; d < kex_cnt[nec]; d++) {
      const int* itab = kex_lists[nec] + (size_t)d * 2 * nec;
      int ncfo = ncf + 1;
      ysaut[ncfo] = 0;
      for (int l = 1; l <= nec; l++) {
        tr_nt[l] = itab[l - 1];
        tr_np[l] = itab[l - 1 + nec];
      }
      transf(nec);
      int mt[12], mp[12];
      for (int l = 1; l <= nec; l++) {
        mt[l] = tr_nt[l];
        mp[l] = tr_np[l];
      }
      (void)mt;
      (void)mp;
      if (ncf < ncfo) continue;
      if (isz != 0) {
        yef1[ncfo] = 1;
      } else {
        int ok = 1;
        for (int l = 1; l <= nec; l++) {
          int ntl = isytr1[tr_nt[l]], npl = isytr1[tr_np[l]];
          if (ntl == 0 || npl == 0) { ok = 0; break; }
          tr_nt[l] = ntl;
          tr_np[l] = npl;
        }
        if (ok) {
          transf(nec);
          if (ncf > ncfo) {
            yef1[ncfo] = 1;
            yef1[ncf] = 1;
            nespo[ncf] = 1;
          }
        }
      }
      if (ncfo >= ncf) continue;
      nesp[ncfo] = ncf - ncfo;
      for (int l = ncfo + 1; l <= ncf; l++) {
        ysaut[l] = 1;
        nesp[l] = 0;
      }
    }
  }
  if (ncf == 0) die("aucun determinant dans le sous espace variationnel");
}

/* ---------------------------------------------- S-space CI (ic001.f:81-131)
   lecdet != 5 with ityper >= 0: H over S (hdig on the diagonal, hntd
   within two excitations, every value kept), its lowest metat eigenpairs
   (the reference calls LAPACK through diagonaliser.f90; restated here by
   cyclic Jacobi rotations).  Each vector's sign: its first component of
   magnitude above 1e-8 of its largest is positive (the reference's signs
   come from LAPACK; E2 and the selection use <I|H|Psi>^2 and do not
   depend on them). */
static void s_space_ci(void) {
  if (metat > ncf) metat = ncf;
  int n = ncf;
  double* a = (double*)xcalloc((size_t)n * n + 4, sizeof(double));
  double* v = (double*)xcalloc((size_t)n * n + 4, sizeof(double));
#define A_(i, j) a[(size_t)((i)-1) * n + ((j)-1)]
#define V_(i, j) v[(size_t)((i)-1) * n + ((j)-1)]
  for (int i = 1; i <= n; i++) {
    hdiag[i] = hdig(i);
    A_(i, i) = hdiag[i];
    V_(i, i) = 1.0;
    for (int j = i + 1; j <= n; j++) {
      int ndif = ne[i] - ne[j];
      for (int k = nd[j] + 1; k <= nd[j] + ne[j]; k++) {
        if (!YOCD(trou[k], i)) ndif++;
        if (!YOCD(part[k], i)) ndif++;
      }
      double h = ndif <= 2 ? hntd(i, j) : 0.0;
      A_(i, j) = A_(j, i) = h;
    }
  }
  double norm = 0.0;
  for (size_t q = 0; q < (size_t)n * n; q++) norm += a[q] * a[q];
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0;
    for (int p = 1; p <= n; p++)
      for (int q = p + 1; q <= n; q++) off += A_(p, q) * A_(p, q);
    if (off <= 1e-30 * norm || off == 0.0) break;
    for (int p = 1; p <= n; p++)
      for (int q = p + 1; q <= n; q++) {
        double apq = A_(p, q);
        if (apq == 0.0) continue;
        double theta = (A_(q, q) - A_(p, p)) / (2.0 * apq);
        double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 1; k <= n; k++) {
          double akp = A_(k, p), akq = A_(k, q);
          A_(k, p) = cs * akp - sn * akq;
          A_(k, q) = sn * akp + cs * akq;
        }
        for (int k = 1; k <= n; k++) {
          double apk = A_(p, k), aqk = A_(q, k);
          A_(p, k) = cs * apk - sn * aqk;
          A_(q, k) = sn * apk + cs * aqk;
        }
        A_(p, q) = A_(q, p) = 0.0;
        for (int k = 1; k <= n; k++) {
          double vkp = V_(k, p), vkq = V_(k, q);
          V_(k, p) = cs * vkp - sn * vkq;
          V_(k, q) = sn * vkp + cs * vkq;
        }
      }
  }
  /* the metat lowest, ascending (ties keep their column order) */
  int* ord = (int*)xcalloc((size_t)n + 4, sizeof(int));
  for (int i = 1; i <= n; i++) ord[i] = i;
  for (int i = 2; i <= n; i++) { /* insertion sort: stable */
    int x = ord[i], j = i - 1;
    while (j >= 1 && A_(ord[j], ord[j]) > A_(x, x)) { ord[j + 1] = ord[j]; j--; }
    ord[j + 1] = x;
  }
  c = (double*)xcalloc((size_t)metat * (size_t)ncf + 4, sizeof(double));
  for (int m = 1; m <= metat; m++) {
    int col = ord[m];
    e[m] = A_(col, col);
    double big = 0.0;
    for (int i = 1; i <= n; i++) if (fabs(V_(i, col)) > big) big = fabs(V_(i, col));
    double sg = 1.0;
    for (int i = 1; i <= n; i++)
      if (fabs(V_(i, col)) > 1e-8 * big) { sg = V_(i, col) < 0.0 ? -1.0 : 1.0; break; }
    for (int i = 1; i <= n; i++) c[(m - 1) * ncf + i] = sg * V_(i, col);
  }
#undef A_
#undef V_
  free(ord);
  free(a);
  free(v);
  printf(" nombre de determinants   ncf=%9d\n valeurs propres\n", ncf);
  for (int m = 1; m <= metat; m++) printf(" %12.8f", e[m]);
  printf("\n");
}

/* ------------------------------------------------------------- unit 4 */
/* brdnee.f:38-135 for ntrsy == 1, isz == 0: the signed index itk(k) of the
   spin-flip image of every determinant of S (0 = none) and the sign itm(m)
   of each root under the flip. */
static int itm_[64];
static void brdnee_itm(void) {
  int* itk = (int*)xcalloc((size_t)ncf + 4, sizeof(int));
  for (int k = 1; k <= ncf; k++) {
    if (ysaut[k]) continue;
    int nespk = nesp[k] + 1, nec = ne[k];
    if (nec == 0) {
      itk[k] = k;
      continue;
    }
    for (int kg = 1; kg <= nespk; kg++) {
      int kk = k + kg - 1, ndk = nd[kk];
      int ntl[16], npl[16], isigne = 1, ncr = 1, ii = kk, ok = 1;
      for (int i = 1; i <= nec; i++) {
        int ntli = isytr1[trou[i + ndk]], npli = isytr1[part[i + ndk]];
        if (ntli == 0 || npli == 0) { ok = 0; break; }
        if (ntli <= 0) isigne = -isigne;
        if (npli <= 0) isigne = -isigne;
        ntl[i] = abs(ntli);
        npl[i] = abs(npli);
      }
      if (!ok) { itk[kk] = 0; continue; }
      int sort = 1;
      if (yef1[k]) {
        int found = 0;
        for (int ig = 1; ig <= nespk; ig++) {
          ii = k + ig - 1;
          int all = 1;
          for (int i = 1; i <= nec && all; i++)
            if (!YOCD(ntl[i], ii) || !YOCD(npl[i], ii)) all = 0;
          if (all) { found = 1; break; }
        }
        if (!found && nec == 1) sort = 0;
      } else {
        ii = kk;
      }
      if (sort) {
        for (int i = 1; i <= nec - 1; i++)
          for (int j = i + 1; j <= nec; j++) {
            if (!(ntl[j] > ntl[i])) { int t = ntl[j]; ntl[j] = ntl[i]; ntl[i] = t; ncr = -ncr; }
            if (!(npl[j] > npl[i])) { int t = npl[j]; npl[j] = npl[i]; npl[i] = t; ncr = -ncr; }
          }
      }
      if (isigne < 0) ii = -ii;
      if (ncr < 0) ii = -ii;
      itk[kk] = ii;
    }
  }
  for (int m = 1; m <= metat; m++) {
    int mncf = (m - 1) * ncf;
    double x = 0.0;
    for (int k = 1; k <= ncf; k++) {
      if (itk[k] == 0) continue;
      int kk = itk[k], ikk = abs(kk);
      double ckk = c[mncf + k] * c[mncf + ikk];
      if (kk < 0) ckk = -ckk;
      x = x + ckk;
    }
    itm_[m] = x < 0.0 ? -1 : 1;
  }
  free(itk);
}

/* cip.f:136-150: zero-order record on unit 4 (rewinds the unit) */
static void write_unit4_zero_order(const char* path, const double* empdet) {
  FILE* f4 = fopen(path, "wb");
  if (!f4) die("cannot rewrite unit 4 file %s", path);
  int jj = ncf * metat, ii = nd[ncf] + ne[ncf] + 1;
  double e0 = ityper == 0 ? escf : 0.0;
  wbuf_t w = {0};
  wb_i4(&w, norb); wb_i4(&w, noca); wb_i4(&w, nocb); wb_i4(&w, metat); wb_i4(&w, ncf); wb_i4(&w, isz);
  unsigned char yb = yion ? 1 : 0;
  wb_put(&w, &yb, 1);
  wb_i4(&w, ii); wb_i4(&w, jj);
  for (int j = 1; j <= ncf; j++) { wb_i4(&w, ne[j]); wb_i4(&w, nd[j]); }
  for (int j = 1; j <= ii; j++) { wb_i4(&w, trou[j]); wb_i4(&w, part[j]); }
  for (int j = 1; j <= jj; j++) wb_r8(&w, c[j]);
  for (int j = 1; j <= metat; j++) wb_r8(&w, e[j] + e0);
  for (int j = 1; j <= metat; j++) wb_r8(&w, emp[j]);
  for (int j = 1; j <= metat; j++) wb_r8(&w, eb[j]);
  for (int j = 1; j <= metat; j++) wb_i4(&w, numero[j]);
  for (int j = 1; j <= ncf; j++) wb_r8(&w, empdet[j]);
  for (int j = 1; j <= norb; j++) wb_r8(&w, fmpb[j]);
  for (int j = 1; j <= norb; j++) wb_r8(&w, tocom[j]);
  /* nblock, nstart (given.f, the S diagonalisation): zero for lecdet = 5 */
  for (int j = 0; j < 2 * UNIT4_NDETZ; j++) wb_i4(&w, 0);
  for (int j = 1; j <= mnorb; j++) wb_i4(&w, iorb[j]);
  for (int j = 1; j <= mnorb; j++) wb_i4(&w, ispin[j]);
  for (int j = 1; j <= ncf; j++)
    for (int i = 1; i <= mnorb; i++) {
      unsigned char y = YOCD(i, j) ? 1 : 0;
      wb_put(&w, &y, 1);
    }
  wb_flush(f4, &w);
  free(w.b);
  fclose(f4);
}

/* the two effective-Hamiltonian records cip appends to unit 4 (hzero with
   escf, ityper and the root signs; then hefmp, hefvp, hefb), from the
   packed triangles hz, hm, hv, hb [1..nbr] */
static void write_unit4_heff(const char* path, const double* hz, const double* hm, const double* hv,
                             const double* hb) {
  FILE* f4 = fopen(path, "ab");
  if (!f4) die("cannot append to unit 4 file %s", path);
  int nbr = metat * (metat + 1) / 2;
  wbuf_t w = {0};
  for (int i = 1; i <= nbr; i++) wb_r8(&w, hz[i]);
  wb_r8(&w, escf);
  wb_i4(&w, ityper);
  wb_i4(&w, ntrsy);
  for (int m = 1; m <= metat; m++) wb_i4(&w, itm_[m]);
  wb_flush(f4, &w);
  free(w.b);
  wbuf_t w2 = {0};
  for (int i = 1; i <= nbr; i++) wb_r8(&w2, hm[i]);
  for (int i = 1; i <= nbr; i++) wb_r8(&w2, hv[i]);
  for (int i = 1; i <= nbr; i++) wb_r8(&w2, hb[i]);
  wb_flush(f4, &w2);
  free(w2.b);
  fclose(f4);
}

/* cip.f:300-306 and 403-414: zero-order and perturbed effective Hamiltonians
   (diagonal: ybrd = .false.) appended to unit 4 */
static void write_unit4_results(const char* path) {
  int nbr = metat * (metat + 1) / 2;
  double* hz = (double*)xcalloc((size_t)nbr + 2, sizeof(double));
  double* hm = (double*)xcalloc((size_t)nbr + 2, sizeof(double));
  double* hv = (double*)xcalloc((size_t)nbr + 2, sizeof(double));
  double* hb = (double*)xcalloc((size_t)nbr + 2, sizeof(double));
  for (int m = 1; m <= metat; m++) {
    int mm = m * (m + 1) / 2;
    double eabs = e[m] + escf;
    hm[mm] = eabs + e2mp[m];
    hv[mm] = eabs + e2vp[m];
    hb[mm] = eabs + e2b[m];
    hz[mm] = eabs - escf;
  }
  write_unit4_heff(path, hz, hm, hv, hb);
  free(hz); free(hm); free(hv); free(hb);
}

/* ------------------------------------------------------------- main */
static char* read_all(FILE* f) {
  size_t cap = 4096, n = 0;
  char* b = (char*)xcalloc(cap, 1);
  int ch;
  while ((ch = fgetc(f)) != EOF) {
    if (n + 2 > cap) {
      cap *= 2;
      b = (char*)realloc(b, cap);
    }
    b[n++] = (char)ch;
  }
  b[n] = 0;
  return b;
}

/* nomfil.f / nomf.f: a non-blank name1 (90 characters) is the file name;
   otherwise the prefix (80 characters) up to its first blank followed by
   the root name (10 characters) up to its first blank -- nothing of the
   root when its 10 characters hold no blank */
static void unit_name(nlgroup_t* g, const char* key, const char* key1, const char* def,
                      const char* prefix, char* out, size_t outsz) {
  const char* v1 = nl_scalar(g, key1);
  if (v1 && strspn(v1, " ") < strlen(v1)) {
    snprintf(out, outsz, "%.90s", v1);
    size_t l = strlen(out);
    while (l && out[l - 1] == ' ') out[--l] = 0;
    return;
  }
  const char* r = nl_scalar(g, key);
  char root[11];
  snprintf(root, sizeof root, "%-10.10s", r ? r : def);
  char* b = strchr(root, ' ');
  if (b) *b = 0;
  else root[0] = 0;
  char pre[81];
  snprintf(pre, sizeof pre, "%.80s", prefix);
  char* pb = strchr(pre, ' ');
  if (pb) *pb = 0;
  snprintf(out, outsz, "%s%s", pre, root);
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ================================================================= moy
 * CIPSI_sources/moy: the Hamiltonian over the determinants read from unit 60
 * (S followed by the selected perturbers), lower triangle row by row, to
 * unit 1 (moy.f:117-199); the determinant lists to units 64 and 61
 * (moy.f:79-104); MP diagonal energies to unit 63 (ystkmp, moy.f:200-208);
 * morue.f: second-order contributions of the determinants beyond the first
 * ndims (the size of S written to unit 4) to unit 33 and a fourth unit-4
 * record.
 *
 * Followed sources: moy/moy.f, moy/openf.f, moy/deter.f (ntrans = 0),
 * moy/lec60.f, moy/transf.f, moy/pie.f, moy/ijkf.f, moy/reijkl.f,
 * moy/hntd.f, moy/hdig.f, moy/hmp.f (the same algorithms as cip's, called
 * here through hntd(), hdig(), hmp() on the moy list), moy/morue.f,
 * moy/stkener.f.  Not restated: yspipro (spin-adapted lists, spipr.f and
 * stk62.f), yion.
 */
#define MOY_LSIZE 8192
#define MOY_NDIMH 10000000

/* moy/lec60.f: the records of unit 60 with vs >= tau, grouped by excitation
   degree (at most 6), the reference determinant counted once */
static void moy_lec60(FILE* f, double tau_) {
  rec_t r = {0};
  rewind(f);
  while (rec_read(f, &r)) {
    int mw = rec_i4(&r), nw = rec_i4(&r);
    int* idet = (int*)xcalloc((size_t)mw + 1, sizeof(int));
    int* necst = (int*)xcalloc((size_t)nw + 1, sizeof(int));
    double* v = (double*)xcalloc((size_t)nw + 1, sizeof(double));
    for (int i = 1; i <= mw; i++) idet[i] = rec_i4(&r);
    for (int i = 1; i <= nw; i++) necst[i] = rec_i4(&r);
    for (int i = 1; i <= nw; i++) v[i] = rec_r8(&r);
    int myy = 0;
    for (int l = 1; l <= nw; l++) {
      int nec = necst[l];
      if (nec > 6) die("erreur degre d excitation %d depasse les possibilites du programme", nec);
      if (v[l] < tau_) {
        myy += 2 * nec;
        continue;
      }
      int itab[20];
      for (int s = 1; s <= nec; s++) {
        itab[s - 1] = idet[++myy];
        itab[s - 1 + nec] = idet[++myy];
      }
      if (nec == 0) {
        if (isz != 0) continue;
        kf_ref++;
        if (kf_ref != 1) {
          kf_ref--;
          printf(" fondamental deja present\n");
        }
        continue;
      }
      kex_push(nec, itab);
    }
    free(idet);
    free(necst);
    free(v);
  }
  free(r.b);
  rewind(f);
}

/* moy/transf.f + moy/pie.f: sort the holes and the particles, check the
   spin orbitals, refuse a determinant of another symmetry, drop a repeat,
   else append it (nd(ncf+1) = nd(ncf) + nec) */
static void moy_transf(int nec) {
  if (nec == 0) {
    ncf++;
    ne[ncf] = 0;
    nd[ncf + 1] = nd[ncf];
    if (isz != 0) ncf--;
    isym = 1;
    return;
  }
  if (nec > 1) {
    for (int i = 1; i <= nec - 1; i++)
      for (int j = i + 1; j <= nec; j++) {
        if (!(tr_nt[j] > tr_nt[i])) { int n = tr_nt[j]; tr_nt[j] = tr_nt[i]; tr_nt[i] = n; }
        if (!(tr_np[j] > tr_np[i])) { int n = tr_np[j]; tr_np[j] = tr_np[i]; tr_np[i] = n; }
      }
  }
  int is = 1, ls = 0;
  if (tr_nt[1] < igela) die("1 spin orbitale est hors de l espace de base");
  if (tr_np[nec] > mnorb) die("1 spin orbitale est hors de l espace de base");
  if (tr_nt[nec] > nocb) die("1 spin orbitale est hors de l espace de base");
  if (tr_np[nec] <= noca) die("1 spin orbitale est hors de l espace de base");
  for (int i = 1; i <= nec; i++) {
    if (!(tr_nt[i] <= noca) && tr_nt[i] < igelb) die("1 spin orbitale est hors de l espace de base");
    if (!(tr_np[i] > nocb)) {
      if (tr_np[i] > norb) die("1 spin orbitale est hors de l espace de base");
      if (tr_np[i] <= noca) die("1 spin orbitale est hors de l espace de base");
    }
    is = its[is][itsym[tr_nt[i]]];
    is = its[is][itsym[tr_np[i]]];
    ls = ls + ispin[tr_np[i]];
    ls = ls - ispin[tr_nt[i]];
  }
  if (isym == 0) isym = is;
  if (is != isym) { /* transf.f:90-95: refused, the run goes on */
    printf(" determinant de mauvaise symetrie\n");
    return;
  }
  if (ls != isz) die("mauvais spin");
  for (int j = ncf; j >= 1; j--) {
    if (ne[j] != nec) continue;
    int d = nd[j], same = 1;
    for (int k = 1; k <= nec; k++)
      if (trou[d + k] != tr_nt[k] || part[d + k] != tr_np[k]) { same = 0; break; }
    if (same) return;
  }
  ncf++;
  if (ncf > g_ncf_cap) die("moy: list capacity exceeded");
  ne[ncf] = nec;
  int d = nd[ncf];
  for (int k = 1; k <= nec; k++) {
    trou[d + k] = tr_nt[k];
    part[d + k] = tr_np[k];
  }
  nd[ncf + 1] = d + nec;
}

/* moy/stkener.f: one (char*40, real*8 x(n)) record appended to unit 33 */
static void moy_stkener(const char* n33, const char* typener, const double* x, int n) {
  FILE* f33 = fopen(n33, "ab");
  if (!f33) die("cannot open unit 33 file %s", n33);
  wbuf_t w = {0};
  char typ[41];
  snprintf(typ, sizeof typ, "%-40.40s", typener);
  wb_put(&w, typ, 40);
  for (int m = 1; m <= n; m++) wb_r8(&w, x[m]);
  wb_flush(f33, &w);
  free(w.b);
  fclose(f33);
  printf(" *************************************\n");
  printf(" %s stockee sur la file 33", typ);
  for (int m = 1; m <= n; m++) printf(" %24.16E", x[m]);
  printf("\n *************************************\n");
}

static void moy_write_buffer(FILE* f1, const int* itab, const int* jtab, const double* vbuf) {
  wbuf_t w = {0};
  for (int k = 1; k <= MOY_LSIZE; k++) wb_i4(&w, itab[k]);
  for (int k = 1; k <= MOY_LSIZE; k++) wb_i4(&w, jtab[k]);
  for (int k = 1; k <= MOY_LSIZE; k++) wb_r8(&w, vbuf[k]);
  wb_flush(f1, &w);
  free(w.b);
}

static int moy_main(const char* json_path) {
  rec_t r = {0};
  /* openf.f */
  nlgroup_t gf;
  static const char* const moyfil_names[] = {"prefix", "det", "ijkl", "f04", "det1", "ijkl1", "f041",
                                             "det_cl", "det_spin", "mat", "enmp", "csf", "det_cl1",
                                             "mat1", "enmp1", "ener", "ener1", "csf1", "det_spin1", NULL};
  nl_parse("moyfil", &gf, moyfil_names);
  char prefix[256] = "";
  {
    const char* v = nl_scalar(&gf, "prefix");
    if (v) snprintf(prefix, sizeof prefix, "%s", v);
  }
  char n01[512], n04[512], n33[512], n40[512], n60[512], n61[512], n63[512], n64[512];
  unit_name(&gf, "mat", "mat1", "mat", prefix, n01, sizeof n01);
  unit_name(&gf, "f04", "f041", "f04", prefix, n04, sizeof n04);
  unit_name(&gf, "ener", "ener1", "ener", prefix, n33, sizeof n33);
  unit_name(&gf, "ijkl", "ijkl1", "ijkl", prefix, n40, sizeof n40);
  unit_name(&gf, "det", "det1", "det", prefix, n60, sizeof n60);
  unit_name(&gf, "det_cl", "det_cl1", "det_cl", prefix, n61, sizeof n61);
  unit_name(&gf, "enmp", "enmp1", "enmp", prefix, n63, sizeof n63);
  unit_name(&gf, "det_spin", "det_spin1", "det_spin", prefix, n64, sizeof n64);

  /* moy.f:50-58: the first record of unit 4 */
  FILE* f4 = fopen(n04, "rb");
  if (!f4) die("cannot open unit 4 file %s", n04);
  if (!rec_read(f4, &r)) die("unit 4: empty");
  norb = rec_i4(&r);
  noca = rec_i4(&r);
  nocb = rec_i4(&r);
  metat = rec_i4(&r);
  int ndet_s = rec_i4(&r);
  isz = rec_i4(&r);
  yion = rec_l1(&r);
  int ii4 = rec_i4(&r), jj4 = rec_i4(&r);
  for (int i = 0; i < 2 * ndet_s + 2 * ii4; i++) (void)rec_i4(&r);
  double* c4 = (double*)xcalloc((size_t)jj4 + 4, sizeof(double)); /* morue.f:29 */
  for (int i = 1; i <= jj4; i++) c4[i] = rec_r8(&r);
  double e4[64], ebmp[64], eben[64];
  if (metat > 60) die("moy: metat > 60");
  for (int m = 1; m <= metat; m++) e4[m] = rec_r8(&r);
  for (int m = 1; m <= metat; m++) ebmp[m] = rec_r8(&r);
  for (int m = 1; m <= metat; m++) eben[m] = rec_r8(&r);
  for (int m = 1; m <= metat; m++) (void)rec_i4(&r);
  for (int i = 1; i <= ndet_s; i++) (void)rec_r8(&r);
  mnorb = 2 * norb;
  fmpb = (double*)xcalloc((size_t)mnorb + 4, sizeof(double));
  for (int i = 1; i <= norb; i++) fmpb[i] = rec_r8(&r);
  for (int i = 1; i <= norb; i++) fmpb[i + norb] = fmpb[i];
  fmpb[mnorb + 1] = 0.0;
  fclose(f4);
  if (yion) die("yion is not restated");

  /* &moyen (moy.f:29-47) */
  int yecr = 0, ystkmp = 0, ymat = 0, yrcmp = 0, y_secd = 0, yspipro = 0;
  double moy_tau = 0.0;
  yprt = 0;
  snprintf(title, sizeof title, "%-20.20s", "");
  nlgroup_t gm;
  static const char* const moyen_names[] = {"yprt", "tau", "yecr", "ystkmp", "ymat", "iord", "title",
                                            "yrcmp", "y_secd", "yspipro", "ysymat", NULL};
  if (!nl_parse("moyen", &gm, moyen_names)) die("erreur dans la namelist moyen");
  nl_set_log(&gm, "yprt", &yprt);
  nl_set_real(&gm, "tau", &moy_tau);
  nl_set_log(&gm, "yecr", &yecr);
  nl_set_log(&gm, "ystkmp", &ystkmp);
  nl_set_log(&gm, "ymat", &ymat);
  nl_set_log(&gm, "yrcmp", &yrcmp);
  nl_set_log(&gm, "y_secd", &y_secd);
  nl_set_log(&gm, "yspipro", &yspipro);
  {
    const char* t = nl_scalar(&gm, "title");
    if (t) snprintf(title, sizeof title, "%-20.20s", t);
  }
  if (yspipro) die("yspipro (spin-adapted lists) is not restated");
  printf(" seuil de selection %10.5f\n", moy_tau);

  /* moy/deter.f: unit 40 header, spin-flip map, the list */
  FILE* f40 = fopen(n40, "rb");
  if (!f40) die("cannot open unit 40 file %s", n40);
  if (!rec_read(f40, &r)) die("empty unit 40");
  nsym = rec_i4(&r);
  int norb40 = rec_i4(&r);
  if (norb40 != norb) die("moy: unit 40 (norb=%d) and unit 4 (norb=%d) differ", norb40, norb);
  (void)rec_i4(&r); /* noc */
  int ntrans = rec_i4(&r);
  itsym = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  for (int i = 1; i <= norb; i++) itsym[i] = itsym[i + norb] = rec_i4(&r);
  (void)rec_i4(&r); /* noa */
  ydp = rec_l1(&r);
  if (ntrans != 0) die("spatial degeneracy operations (ntrans>0) are not restated");
  if (!rec_read(f40, &r)) die("unit 40: missing its");
  for (int j = 1; j <= nsym; j++)
    for (int i = 1; i <= nsym; i++) its[i][j] = rec_i4(&r);
  igela = 1;
  igelb = igela + norb;
  iorb = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  ispin = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  isytr1 = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  for (int i = 1; i <= norb; i++) {
    iorb[i] = i;
    iorb[i + norb] = i;
    ispin[i] = 0;
    ispin[i + norb] = 1;
  }
  for (int i = 1; i <= norb; i++) {
    int k = i + norb, zero = 0;
    if (k < igelb && i > igela) zero = 1;
    if (k > igelb && i < igela) zero = 1;
    if (k < nocb && i > noca) zero = 1;
    if (k > nocb && i < noca) zero = 1;
    isytr1[i] = zero ? 0 : k;
    isytr1[k] = zero ? 0 : i;
  }
  FILE* fd60 = fopen(n60, "rb");
  if (!fd60) die("cannot open unit 60 file %s", n60);
  moy_lec60(fd60, moy_tau);
  fclose(fd60);
  {
    long long tot = 2, ntp = 2;
    for (int nec = 1; nec <= 6; nec++) {
      tot += kex_cnt[nec];
      ntp += (long long)kex_cnt[nec] * nec;
    }
    g_ncf_cap = (int)(2 * tot + 4);
    ntp_cap = (int)(2 * ntp + 64);
  }
  ne = (int*)xcalloc((size_t)g_ncf_cap + 4, sizeof(int));
  nd = (int*)xcalloc((size_t)g_ncf_cap + 4, sizeof(int));
  trou = (int*)xcalloc((size_t)ntp_cap + 64, sizeof(int));
  part = (int*)xcalloc((size_t)ntp_cap + 64, sizeof(int));
  ncf = 0;
  isym = 0;
  if (kf_ref) moy_transf(0);
  for (int nec = 1; nec <= 6; nec++) {
    for (int d = 0; d < kex_cnt[nec]; d++) {
      const int* itab = kex_lists[nec] + (size_t)d * 2 * nec;
      int ncfo = ncf + 1;
      for (int l = 1; l <= nec; l++) {
        tr_nt[l] = itab[l - 1];
        tr_np[l] = itab[l - 1 + nec];
      }
      moy_transf(nec);
      if (ncf < ncfo) continue;
      if (isz != 0) continue;
      int ok = 1;
      for (int l = 1; l <= nec; l++) {
        int ntl = isytr1[tr_nt[l]], npl = isytr1[tr_np[l]];
        if (ntl == 0 || npl == 0) { ok = 0; break; }
        tr_nt[l] = ntl;
        tr_np[l] = npl;
      }
      if (ok) moy_transf(nec);
    }
  }
  printf(" determinants engendres\n%12d\n", ncf);
  if (ncf > MOY_NDIMH) die("moy: stop 99 (more than %d determinants)", MOY_NDIMH);

  /* moy.f:79-104: units 64 and 61 */
  {
    int ii = nd[ncf] + ne[ncf] + 1;
    FILE* f64 = fopen(n64, "wb");
    if (!f64) die("cannot open unit 64 file %s", n64);
    wbuf_t w = {0};
    wb_i4(&w, ncf);
    wb_i4(&w, ii);
    wb_i4(&w, mnorb);
    unsigned char yb = 0;
    wb_put(&w, &yb, 1);
    for (int i = 1; i <= ncf; i++) { wb_i4(&w, ne[i]); wb_i4(&w, nd[i]); }
    for (int i = 1; i <= ii; i++) { wb_i4(&w, trou[i]); wb_i4(&w, part[i]); }
    for (int i = 1; i <= mnorb + 1; i++) wb_i4(&w, i <= mnorb ? iorb[i] : 0);
    for (int i = 1; i <= mnorb + 1; i++) wb_i4(&w, i <= mnorb ? ispin[i] : 0);
    wb_flush(f64, &w);
    free(w.b);
    fclose(f64);
    FILE* f61 = fopen(n61, "wb");
    if (!f61) die("cannot open unit 61 file %s", n61);
    for (int i = 1; i <= ncf; i++) {
      wbuf_t a = {0};
      wb_i4(&a, ne[i]);
      wb_flush(f61, &a);
      free(a.b);
      if (ne[i] != 0) {
        wbuf_t b = {0};
        for (int j = 1; j <= ne[i]; j++) wb_i4(&b, trou[nd[i] + j]);
        for (int j = 1; j <= ne[i]; j++) wb_i4(&b, part[nd[i] + j]);
        wb_flush(f61, &b);
        free(b.b);
      }
    }
    fclose(f61);
  }
  if (yrcmp) { /* moy.f:106-107: the lists only */
    fclose(f40);
    FILE* fj = fopen(json_path, "w");
    if (fj) {
      fprintf(fj, "{\"ncf\": %d, \"ndims\": %d, \"yrcmp\": true, \"variant\": \"moy\"}\n", ncf, ndet_s);
      fclose(fj);
    }
    return 0;
  }

  /* moy/ijkf.f (no zeroing of small Fock elements) and moy/reijkl.f */
  int nter = norb * (norb + 1) / 2;
  f_ = (double*)xcalloc((size_t)nter + 4, sizeof(double));
  aj = (double*)xcalloc((size_t)nter + 4, sizeof(double));
  ak = (double*)xcalloc((size_t)nter + 4, sizeof(double));
  fdiag = (double*)xcalloc((size_t)mnorb + 4, sizeof(double));
  if (!rec_read(f40, &r)) die("unit 40: missing h");
  if (!rec_read(f40, &r)) die("unit 40: missing J");
  for (int l = 1; l <= nter; l++) aj[l] = rec_r8(&r);
  if (!rec_read(f40, &r)) die("unit 40: missing K");
  for (int l = 1; l <= nter; l++) ak[l] = rec_r8(&r);
  if (!rec_read(f40, &r)) die("unit 40: missing F");
  for (int l = 1; l <= nter; l++) f_[l] = rec_r8(&r);
  {
    int l = 0;
    for (int ll = 1; ll <= norb; ll++) {
      l += ll;
      fdiag[ll] = f_[l];
      fdiag[ll + norb] = f_[l];
    }
  }
  ij0_ = (int16_t*)xcalloc((size_t)norb * (size_t)norb, sizeof(int16_t));
  if (!rec_read(f40, &r)) die("unit 40: missing ij0");
  for (int j = 1; j <= norb; j++)
    for (int i = 1; i <= norb; i++) IJ0(i, j) = rec_i2(&r);
  if (!rec_read(f40, &r)) die("unit 40: missing ninte");
  ninte = rec_i4(&r);
  for (int i = 1; i <= nsym; i++) ntttt[i] = rec_i4(&r);
  {
    long long lsize = 8192, nbuf = ninte / lsize + 1, mint = 0;
    bijkl = (float*)xcalloc((size_t)(nbuf * lsize) + 4, sizeof(float));
    for (long long k = 0; k < nbuf; k++) {
      if (!rec_read(f40, &r)) die("unit 40: missing integral buffer %lld", k + 1);
      for (long long i = 0; i < lsize; i++) {
        ++mint;
        bijkl[mint] = ydp ? (float)rec_r8(&r) : rec_r4(&r);
      }
    }
  }
  fclose(f40);

  /* moy.f:117-199: the matrix, row by row, to unit 1 */
  static int itab[MOY_LSIZE + 1], jtab[MOY_LSIZE + 1];
  static double vbuf[MOY_LSIZE + 1];
  double* stefen = (double*)xcalloc((size_t)ncf + 4, sizeof(double));
  double* stefmp = (double*)xcalloc((size_t)ncf + 4, sizeof(double));
  unsigned char* yocm = (unsigned char*)xcalloc((size_t)mnorb + 4, 1);
  FILE* f1 = fopen(n01, "wb");
  if (!f1) die("cannot open unit 1 file %s", n01);
  long long nhntd = 0, nhij = 0, nrec1 = 0;
  int nbuf = 0;
  const double th0 = now_s();
  for (int i = 1; i <= ncf; i++) {
    int ne1 = ne[i];
    for (int k = 1; k <= ne1; k++) {
      yocm[trou[nd[i] + k]] = 1;
      yocm[part[nd[i] + k]] = 1;
    }
    int im1 = i - 1;
    if (y_secd && im1 > ndet_s) im1 = ndet_s;
    for (int j = 1; j <= im1; j++) {
      int ne2 = ne[j];
      int ndif = ne1 - ne2;
      if (ndif > 2) continue;
      if (ne2 != 0) {
        for (int k = 1; k <= ne2; k++) {
          if (!yocm[trou[nd[j] + k]]) ndif++;
          if (!yocm[part[nd[j] + k]]) ndif++;
        }
        if (ndif > 2) continue;
      }
      double hij = hntd(i, j);
      nhntd++;
      if (fabs(hij) < 1.0e-10) continue;
      nhij++;
      nbuf++;
      itab[nbuf] = i;
      jtab[nbuf] = j;
      vbuf[nbuf] = hij;
      if (nbuf < MOY_LSIZE) continue;
      moy_write_buffer(f1, itab, jtab, vbuf);
      nrec1++;
      nbuf = 0;
    }
    double stfn = hdig(i);
    nhntd++;
    nhij++;
    stefen[i] = stfn;
    stefmp[i] = hmp(i);
    nbuf++;
    itab[nbuf] = i;
    jtab[nbuf] = i;
    vbuf[nbuf] = stfn * 0.5;
    if (nbuf >= MOY_LSIZE) {
      moy_write_buffer(f1, itab, jtab, vbuf);
      nrec1++;
      nbuf = 0;
    }
    for (int k = 1; k <= ne1; k++) {
      yocm[trou[nd[i] + k]] = 0;
      yocm[part[nd[i] + k]] = 0;
    }
  }
  itab[MOY_LSIZE] = -1;
  jtab[MOY_LSIZE] = nbuf;
  moy_write_buffer(f1, itab, jtab, vbuf);
  nrec1++;
  fclose(f1);
  const double hloop_s = now_s() - th0;
  if (nbuf == 0) printf(" **** attention le dernier buffer sur 1 ne contient aucun element\n");
  printf(" *** fin de la construction de h ***\n appels a hntd %10lld elements stockes sur 1 %10lld\n",
         nhntd, nhij);
  if (ystkmp) {
    FILE* f63 = fopen(n63, "wb");
    if (!f63) die("cannot open unit 63 file %s", n63);
    wbuf_t w = {0};
    for (int i = 1; i <= ncf; i++) wb_r8(&w, stefmp[i]);
    wb_flush(f63, &w);
    free(w.b);
    fclose(f63);
  }

  /* morue.f: second order of the determinants k > ndims on the roots of S,
     from the unit-1 elements (k, i <= ndims) of each row k */
  int mmm = metat * (metat + 1) / 2;
  double* hefmp = (double*)xcalloc((size_t)mmm + 2, sizeof(double));
  double* hefen = (double*)xcalloc((size_t)mmm + 2, sizeof(double));
  double* hefenb = (double*)xcalloc((size_t)mmm + 2, sizeof(double));
  double cunt[64];
  for (int m = 1; m <= metat; m++) cunt[m] = 0.0;
  int ndims = ndet_s;
  if (ndims != ncf) {
    f1 = fopen(n01, "rb");
    if (!f1) die("cannot reopen unit 1 file %s", n01);
    static int rt[MOY_LSIZE + 1], rj[MOY_LSIZE + 1];
    static double rv[MOY_LSIZE + 1];
    int last = MOY_LSIZE, nb = MOY_LSIZE;
    rt[MOY_LSIZE] = 0;
    for (;;) {
      nb++;
      if (nb > last) {
        if (rt[MOY_LSIZE] == -1) break;
        if (!rec_read(f1, &r)) die("unit 1: missing record");
        for (int k = 1; k <= MOY_LSIZE; k++) rt[k] = rec_i4(&r);
        for (int k = 1; k <= MOY_LSIZE; k++) rj[k] = rec_i4(&r);
        for (int k = 1; k <= MOY_LSIZE; k++) rv[k] = rec_r8(&r);
        if (rt[MOY_LSIZE] == -1) last = rj[MOY_LSIZE];
        nb = 1;
      }
      int k = rt[nb], i = rj[nb];
      if (k == 1) continue;
      if (k == i && k > ndims) {
        double stenk = stefen[k], stmpk = stefmp[k];
        double enk2 = stenk + stenk, empk2 = stmpk + stmpk;
        int ii = 0;
        for (int m = 1; m <= metat; m++)
          for (int n = 1; n <= m; n++) {
            ii++;
            double denb = eben[m] + eben[n] - enk2;
            double dmp = ebmp[m] + ebmp[n] - empk2;
            double den = e4[m] + e4[n] - enk2;
            double hmn = cunt[m] * cunt[n];
            hmn = hmn + hmn;
            hefmp[ii] = hefmp[ii] + hmn / dmp;
            hefen[ii] = hefen[ii] + hmn / den;
            hefenb[ii] = hefenb[ii] + hmn / denb;
          }
        for (int m = 1; m <= metat; m++) cunt[m] = 0.0;
        continue;
      }
      if (k <= ndims || i > ndims) continue;
      double hij = rv[nb];
      int mi = i - ndims;
      for (int m = 1; m <= metat; m++) {
        mi = mi + ndims;
        cunt[m] = cunt[m] + c4[mi] * hij;
      }
    }
    fclose(f1);
    char typener[96];
    for (int m = 1; m <= metat; m++) cunt[m] = hefmp[m * (m + 1) / 2];
    snprintf(typener, sizeof typener, "moyens mbp %s", title);
    moy_stkener(n33, typener, cunt, metat);
    for (int m = 1; m <= metat; m++) cunt[m] = hefen[m * (m + 1) / 2];
    snprintf(typener, sizeof typener, "moyens envp%s", title);
    moy_stkener(n33, typener, cunt, metat);
    for (int m = 1; m <= metat; m++) cunt[m] = hefenb[m * (m + 1) / 2];
    snprintf(typener, sizeof typener, "moyens enb %s", title);
    moy_stkener(n33, typener, cunt, metat);
  }
  /* morue.f:8300: the fourth record of unit 4 replaces whatever follows the
     third (ny, never set in morue, is written as 0) */
  {
    f4 = fopen(n04, "rb");
    if (!f4) die("cannot reopen unit 4 file %s", n04);
    long keep = 0;
    for (int q = 0; q < 3; q++) {
      if (!rec_read(f4, &r)) die("unit 4: fewer than three records");
      keep = ftell(f4);
    }
    fclose(f4);
    if (truncate(n04, keep) != 0) die("cannot truncate unit 4 file %s", n04);
    f4 = fopen(n04, "ab");
    if (!f4) die("cannot append to unit 4 file %s", n04);
    wbuf_t w = {0};
    for (int i = 1; i <= mmm; i++) wb_r8(&w, hefmp[i]);
    for (int i = 1; i <= mmm; i++) wb_r8(&w, hefen[i]);
    for (int i = 1; i <= mmm; i++) wb_r8(&w, hefenb[i]);
    wb_i4(&w, 0);
    wb_flush(f4, &w);
    free(w.b);
    fclose(f4);
  }

  FILE* fj = fopen(json_path, "w");
  if (fj) {
    fprintf(fj, "{\n  \"ncf\": %d, \"ndims\": %d, \"metat\": %d, \"norb\": %d,\n", ncf, ndims, metat, norb);
    fprintf(fj, "  \"nhntd\": %lld, \"nhij\": %lld, \"unit1_records\": %lld,\n", nhntd, nhij, nrec1);
    fprintf(fj, "  \"hloop_s\": %.6f,\n", hloop_s);
    const char* nm[3] = {"hefmp", "hefen", "hefenb"};
    double* ar[3] = {hefmp, hefen, hefenb};
    for (int q = 0; q < 3; q++) {
      fprintf(fj, "  \"%s\": [", nm[q]);
      for (int i = 1; i <= mmm; i++) fprintf(fj, "%s%.17g", i > 1 ? ", " : "", ar[q][i]);
      fprintf(fj, "],\n");
    }
    fprintf(fj, "  \"variant\": \"moy\"\n}\n");
    fclose(fj);
  }
  free(r.b);
  return 0;
}

static void usage(void) {
  fprintf(stderr,
          "usage: cipsi_ref [--sym] [--json out.json] [--candlog file] [--genmask file]\n"
          "                 [--no-pertu-ref] [--sample M --plan file] < stdin-namelists\n"
          "       cipsi_ref --moy [--json out.json] < stdin-namelists   (moy: H over unit 60)\n"
          "  --plan: lines 'm k1 k2 ...' (1-based generators); each line runs those\n"
          "  generators on the sample residue m and reports [perturbers, seconds]\n");
  exit(2);
}

int main(int argc, char** argv) {
  const char* json_path = "cipsi_ref.json";
  const char* cand_path = NULL;
  const char* mask_path = NULL;
  const char* plan_path = NULL;
  int run_moy = 0;
  for (int a = 1; a < argc; a++) {
    if (!strcmp(argv[a], "--sym"))
      g_sym_variant = 1;
    else if (!strcmp(argv[a], "--json") && a + 1 < argc)
      json_path = argv[++a];
    else if (!strcmp(argv[a], "--candlog") && a + 1 < argc)
      cand_path = argv[++a];
    else if (!strcmp(argv[a], "--genmask") && a + 1 < argc)
      mask_path = argv[++a];
    else if (!strcmp(argv[a], "--no-pertu-ref"))
      run_pertu_ref = 0;
    else if (!strcmp(argv[a], "--sample") && a + 1 < argc)
      samp_M = atoll(argv[++a]);
    else if (!strcmp(argv[a], "--plan") && a + 1 < argc)
      plan_path = argv[++a];
    else if (!strcmp(argv[a], "--moy"))
      run_moy = 1;
    else
      usage();
  }
  g_stdin_text = read_all(stdin);
  if (run_moy) return moy_main(json_path);

  /* openf.f */
  nlgroup_t gf;
  static const char* const cipfil_names[] = {"prefix", "det", "ijkl", "f04", "det1", "ijkl1", "f041",
                                             "ocno1", "bdvec", "bdvec1", "ocno", "ener", "ener1", NULL};
  nl_parse("cipfil", &gf, cipfil_names);
  char prefix[256] = "";
  {
    const char* v = nl_scalar(&gf, "prefix");
    if (v) snprintf(prefix, sizeof prefix, "%s", v);
  }
  char n60[512], n40[512], n04[512], n21[512], n59[512], n33[512];
  unit_name(&gf, "det", "det1", "det", prefix, n60, sizeof n60);
  unit_name(&gf, "ijkl", "ijkl1", "ijkl", prefix, n40, sizeof n40);
  unit_name(&gf, "f04", "f041", "f04", prefix, n04, sizeof n04);
  unit_name(&gf, "ocno", "ocno1", "ocno", prefix, n21, sizeof n21);
  unit_name(&gf, "bdvec", "bdvec1", "bdvec", prefix, n59, sizeof n59);
  unit_name(&gf, "ener", "ener1", "ener", prefix, n33, sizeof n33);

  FILE* f40 = fopen(n40, "rb");
  if (!f40) die("cannot open unit 40 file %s", n40);

  /* deter.f: header of unit 40 */
  rec_t r = {0};
  if (!rec_read(f40, &r)) die("empty unit 40");
  nsym = rec_i4(&r);
  norb = rec_i4(&r);
  hf_noc = rec_i4(&r);
  int ntrans = rec_i4(&r);
  int* itsyp = (int*)xcalloc((size_t)norb * 2 + 4, sizeof(int));
  for (int i = 1; i <= norb; i++) itsyp[i] = rec_i4(&r);
  (void)rec_i4(&r); /* noa */
  ydp = rec_l1(&r);
  if (ntrans != 0) die("spatial degeneracy operations (ntrans>0) are not restated");
  if (!rec_read(f40, &r)) die("unit 40: missing its");
  for (int j = 1; j <= nsym; j++)
    for (int i = 1; i <= nsym; i++) its[i][j] = rec_i4(&r);
  mnorb = 2 * norb;
  /* spin orbital tables */
  fdiag = (double*)xcalloc((size_t)mnorb + 4, sizeof(double));
  tocom = (double*)xcalloc((size_t)mnorb + 4, sizeof(double));
  fmpb = (double*)xcalloc((size_t)mnorb + 4, sizeof(double));
  ispin = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  iorb = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  itsym = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  yoc = (unsigned char*)xcalloc((size_t)mnorb + 4, 1);
  yocs = (unsigned char*)xcalloc((size_t)mnorb + 4, 1);
  isytr1 = (int*)xcalloc((size_t)mnorb + 4, sizeof(int));
  yorper = (unsigned char*)xcalloc((size_t)norb + 4, 1);
  for (int i = 1; i <= norb; i++) {
    itsym[i] = itsyp[i];
    itsym[i + norb] = itsyp[i];
  }

  /* defaults (deter.f:78-226) */
  ntrsy = 1;
  ytoul = 1; yion = 0; isym = 0; isz = 0; test = 0.5; teseff = -1.0; yprt = 0; ybrd = 0;
  for (int i = 1; i <= hf_noc; i++) tocom[i] = 2.0;
  escf = 0.0; ystkic = 0; ityper = 1;
  aval[1] = 0.128e-6; aval[2] = 0.64e-6; aval[3] = 0.32e-5; aval[4] = 0.16e-4;
  aval[5] = 0.8e-4; aval[6] = 0.4e-3; aval[7] = 0.2e-2; aval[8] = 0.1e-1; aval[9] = 0.5e-1;
  aval[10] = 1.0;
  ywvi = 0; ywvf = 1; ndiag = 6; tau = 1.0e-4; ytocom = 0; ypertu = 1; ymoyen = 0;
  iselec = 1; lecdet = 1; nclass = 10; metat = 1; ywdeg = 1; coeff = 0.0; ninact = 0;
  maxdet = 500000; twdet = 0.0;
  for (int i = 1; i <= 60; i++) numero[i] = i;
  for (int i = 1; i <= norb; i++) numac[i] = i; /* deter.f:139 */
  noac = 0; nusym = 1; nelac = 0; nemax = 8;
  nlgroup_t gi;
  /* deter.f:52-58 (cipsym adds nemax) */
  static const char* const icinp_names[] = {
      "test", "ndiag", "isz", "metat", "tocom", "yprt", "yion", "ybrd", "ityper", "numero", "coeff",
      "ygen", "title", "tau", "ymoyen", "aval", "nclass", "ytoul", "lecdet", "tdet", "maxdet", "teseff",
      "nvr", "numac", "nelac", "nusym", "noac", "ywvi", "ywvf", "ystkic", "ywdeg", "ytocom", "iselec",
      "iord", "twdet", "mspin", "ydp", "ninact", "nonact", "nemax", NULL};
  static const char* const icinp_names_cip[] = {
      "test", "ndiag", "isz", "metat", "tocom", "yprt", "yion", "ybrd", "ityper", "numero", "coeff",
      "ygen", "title", "tau", "ymoyen", "aval", "nclass", "ytoul", "lecdet", "tdet", "maxdet", "teseff",
      "nvr", "numac", "nelac", "nusym", "noac", "ywvi", "ywvf", "ystkic", "ywdeg", "ytocom", "iselec",
      "iord", "twdet", "mspin", "ydp", "ninact", "nonact", NULL};
  if (!nl_parse("icinp", &gi, g_sym_variant ? icinp_names : icinp_names_cip))
    die("erreur dans la namelist icinp");
  nl_set_real(&gi, "test", &test);
  nl_set_int(&gi, "ndiag", &ndiag);
  nl_set_int(&gi, "isz", &isz);
  nl_set_int(&gi, "metat", &metat);
  nl_set_real_arr(&gi, "tocom", tocom + 1, norb, 512);
  nl_set_log(&gi, "yprt", &yprt);
  nl_set_log(&gi, "yion", &yion);
  nl_set_log(&gi, "ybrd", &ybrd);
  nl_set_int(&gi, "ityper", &ityper);
  nl_set_int_arr(&gi, "numero", numero + 1, 60, 60);
  nl_set_real(&gi, "coeff", &coeff);
  nl_set_real(&gi, "tau", &tau);
  nl_set_log(&gi, "ymoyen", &ymoyen);
  nl_set_real_arr(&gi, "aval", aval + 1, 10, 10);
  nl_set_int(&gi, "nclass", &nclass);
  nl_set_log(&gi, "ytoul", &ytoul);
  nl_set_int(&gi, "lecdet", &lecdet);
  nl_set_real(&gi, "tdet", &tdet);
  nl_set_int(&gi, "maxdet", &maxdet);
  nl_set_real(&gi, "teseff", &teseff);
  nl_set_log(&gi, "ywvi", &ywvi);
  nl_set_log(&gi, "ywvf", &ywvf);
  nl_set_log(&gi, "ystkic", &ystkic);
  nl_set_log(&gi, "ywdeg", &ywdeg);
  nl_set_log(&gi, "ytocom", &ytocom);
  nl_set_int(&gi, "iselec", &iselec);
  nl_set_real(&gi, "twdet", &twdet);
  nl_set_int(&gi, "ninact", &ninact);
  {
    const char* t = nl_scalar(&gi, "title");
    if (t) snprintf(title, sizeof title, "%-20.20s", t);
  }
  nl_set_log(&gi, "ydp", &ydp); /* after the unit-40 header (deter.f:119,222) */
  int nonact[512] = {0};
  nl_set_int_arr(&gi, "nonact", nonact, 512, 512);
  {
    int ms[64];
    nl_set_int_arr(&gi, "mspin", ms, 0, 60);
  }
  if (nl_get(&gi, "ygen")) die("ygen given in the namelist is not restated");
  if (nl_get(&gi, "iord")) die("iord given in the namelist is not restated");
  nl_set_int(&gi, "noac", &noac);
  nl_set_int(&gi, "nelac", &nelac);
  nl_set_int(&gi, "nusym", &nusym);
  if (g_sym_variant) nl_set_int(&gi, "nemax", &nemax);
  nl_set_int_arr(&gi, "numac", numac + 1, 512, 512);

  if (teseff < 0.0) teseff = 0.05 * tau;
  if (lecdet == 5) tdet = 0.0;
  if (ytocom) { /* deter.f:228-229: occupations of the Fock operator from unit 21 */
    FILE* f21 = fopen(n21, "rb");
    if (!f21) die("cannot open unit 21 file %s", n21);
    rec_t r21 = {0};
    if (!rec_read(f21, &r21)) die("unit 21: no occupation record");
    for (int i = 1; i <= norb; i++) tocom[i] = rec_r8(&r21);
    free(r21.b);
    fclose(f21);
  }
  if (ityper == 0) ypertu = 0;
  if (ityper == 1) yen = 0;
  if (ityper == 2) yen = 1;
  if (iselec == 1) yselm = 1;
  if (iselec == 2) yselm = 0;
  if (iselec == 3) ysele = 1;
  if (yion) die("yion is not restated");
  if (ybrd && metat > 1) die("ybrd (QDPT heff) is not restated");
  if (lecdet < 2 || lecdet > 5) die("lecdet=%d is not restated", lecdet);
  if (metat > 60) die("trop d etats demandes en perturbation");

  noca = 0; nocb = 0; igela = 0; igelb = 0;
  /* deter.f:241-251 */
  if (noca == 0) {
    if (nocb == 0) nocb = hf_noc;
    noca = nocb;
    nocb = nocb + norb;
  }
  igela = igela + 1;
  if (igelb < norb) igelb = igela + norb;
  for (int i = 1; i <= norb; i++) {
    iorb[i] = i;
    iorb[i + norb] = i;
    ispin[i] = 0;
    ispin[i + norb] = 1;
  }
  for (int i = 1; i <= norb; i++) {
    int k = i + norb;
    int zero = 0;
    if (k < igelb && i > igela) zero = 1;
    if (k > igelb && i < igela) zero = 1;
    if (k < nocb && i > noca) zero = 1;
    if (k > nocb && i < noca) zero = 1;
    isytr1[i] = zero ? 0 : k;
    isytr1[k] = zero ? 0 : i;
  }
  noc_[1] = noca; noc_[2] = nocb;
  igels_[1] = igela; igels_[2] = igelb;
  norbs_[1] = norb; norbs_[2] = mnorb;
  for (int i = 1; i <= norb; i++) yorper[i] = 1;
  if (ninact > 0) {
    yreduc = 1;
    for (int i = 0; i < ninact; i++) yorper[nonact[i]] = 0;
  }

  /* S: lec60 (lecdet 2, 3, 5) or cas (lecdet 4), then the spin-flip closure */
  if (lecdet == 4) {
    cas();
  } else {
    f60 = fopen(n60, "rb");
    if (!f60) die("cannot open unit 60 file %s", n60);
    lec60(f60);
    fclose(f60);
    f60 = NULL;
  }
  {
    long long tot = 1, ntp = 2;
    for (int nec = 1; nec <= 8; nec++) {
      tot += kex_cnt[nec];
      ntp += (long long)kex_cnt[nec] * nec;
    }
    g_ncf_cap = (int)(2 * tot + 4);
    ntp_cap = (int)(2 * ntp + 64);
  }
  ne = (int*)xcalloc((size_t)g_ncf_cap + 4, sizeof(int));
  nd = (int*)xcalloc((size_t)g_ncf_cap + 4, sizeof(int));
  trou = (int*)xcalloc((size_t)ntp_cap + 64, sizeof(int));
  part = (int*)xcalloc((size_t)ntp_cap + 64, sizeof(int));
  ygen = (unsigned char*)xcalloc((size_t)g_ncf_cap + 4, 1);
  ysaut = (unsigned char*)xcalloc((size_t)g_ncf_cap + 4, 1);
  yef1 = (unsigned char*)xcalloc((size_t)g_ncf_cap + 4, 1);
  nesp = (int*)xcalloc((size_t)g_ncf_cap + 4, sizeof(int));
  nespo = (int*)xcalloc((size_t)g_ncf_cap + 4, sizeof(int));
  hdiag = (double*)xcalloc((size_t)g_ncf_cap + 4, sizeof(double));
  yocd_ld = mnorb + 2;
  yocd_ = (unsigned char*)xcalloc((size_t)(g_ncf_cap + 4) * (size_t)yocd_ld, 1);
  build_space();
  printf(" determinants lus, ncf= %d\n", ncf);
  nesp[ncf] = 0; /* cip.f:55 */
  noc1 = noca > nocb - norb ? noca : nocb - norb;
  noc2 = noca < nocb - norb ? noca : nocb - norb;

  /* ijkf.f */
  int nter = norb * (norb + 1) / 2;
  f_ = (double*)xcalloc((size_t)nter + 4, sizeof(double));
  aj = (double*)xcalloc((size_t)nter + 4, sizeof(double));
  ak = (double*)xcalloc((size_t)nter + 4, sizeof(double));
  if (!rec_read(f40, &r)) die("unit 40: missing h");
  if (!rec_read(f40, &r)) die("unit 40: missing J");
  for (int l = 1; l <= nter; l++) aj[l] = rec_r8(&r);
  if (!rec_read(f40, &r)) die("unit 40: missing K");
  for (int l = 1; l <= nter; l++) ak[l] = rec_r8(&r);
  if (!rec_read(f40, &r)) die("unit 40: missing F");
  for (int l = 1; l <= nter; l++) f_[l] = rec_r8(&r);
  for (int i = 1; i <= norb; i++)
    for (int j = 1; j <= i; j++)
      if (fabs(f_[i * (i - 1) / 2 + j]) < 1.0e-10) f_[i * (i - 1) / 2 + j] = 0.0;
  {
    int l = 0;
    for (int ll = 1; ll <= norb; ll++) {
      l += ll;
      fdiag[ll] = f_[l];
      fdiag[ll + norb] = f_[l];
    }
  }
  /* reijkl.f */
  ij0_ = (int16_t*)xcalloc((size_t)norb * (size_t)norb, sizeof(int16_t));
  if (!rec_read(f40, &r)) die("unit 40: missing ij0");
  for (int j = 1; j <= norb; j++)
    for (int i = 1; i <= norb; i++) IJ0(i, j) = rec_i2(&r);
  if (!rec_read(f40, &r)) die("unit 40: missing ninte");
  ninte = rec_i4(&r);
  for (int i = 1; i <= nsym; i++) ntttt[i] = rec_i4(&r);
  {
    long long lsize = 8192, nbuf = ninte / lsize + 1, mint = 0;
    bijkl = (float*)xcalloc((size_t)(nbuf * lsize) + 4, sizeof(float));
    for (long long k = 0; k < nbuf; k++) {
      if (!rec_read(f40, &r)) die("unit 40: missing integral buffer %lld", k + 1);
      for (long long i = 0; i < lsize; i++) {
        ++mint;
        bijkl[mint] = ydp ? (float)rec_r8(&r) : rec_r4(&r);
      }
    }
  }
  fclose(f40);

  /* rdener.f: escf */
  {
    FILE* f33 = fopen(n33, "rb");
    if (!f33) die("cannot open unit 33 file %s", n33);
    int found = 0;
    while (rec_read(f33, &r)) {
      if (r.len >= 40 && strncmp((char*)r.b, "energie du determinant de reference     ", 40) == 0) {
        r.pos = 40;
        int jv = rec_i4(&r);
        if (jv < 1) die("bad escf record");
        escf = rec_r8(&r);
        found = 1;
        break;
      }
    }
    fclose(f33);
    if (!found) die("energie du determinant de reference n'existe pas sur 33");
  }

  /* ic001.f:44-76 (ynoic, lecdet=5); not called when ityper < 0
     (cip.f:71), which leaves c and e at zero */
  if (ityper < 0) {
    c = (double*)xcalloc((size_t)metat * (size_t)ncf + 4, sizeof(double));
  } else if (lecdet != 5) {
    s_space_ci();
  } else {
    FILE* f4 = fopen(n04, "rb");
    if (!f4) die("cannot open unit 4 file %s", n04);
    if (!rec_read(f4, &r)) die("unit 4: empty");
    (void)rec_i4(&r); (void)rec_i4(&r); (void)rec_i4(&r); (void)rec_i4(&r);
    int mcf = rec_i4(&r);
    int* iord60 = (int*)xcalloc((size_t)mcf + 4, sizeof(int));
    if (!g_sym_variant) {
      if (!rec_read(f4, &r)) die("unit 4: missing iord60");
      for (int k = 1; k <= mcf; k++) iord60[k] = rec_i4(&r);
    }
    fclose(f4);
    FILE* f59 = fopen(n59, "rb");
    if (!f59) die("cannot open unit 59 file %s", n59);
    if (!rec_read(f59, &r)) die("unit 59: empty");
    int ncf59 = rec_i4(&r);
    int met59 = rec_i4(&r);
    if (ncf59 != ncf) die("files 59 (ncf=%d) and S (ncf=%d) incompatible", ncf59, ncf);
    metat = met59;
    if (metat > 60) die("trop d etats demandes en perturbation");
    c = (double*)xcalloc((size_t)metat * (size_t)ncf + 4, sizeof(double));
    for (int i = 1; i <= metat * ncf; i++) c[i] = rec_r8(&r);
    for (int i = 1; i <= metat; i++) e[i] = rec_r8(&r);
    fclose(f59);
    for (int i = 1; i <= metat; i++) e[i] = e[i] - escf;
    if (mcf != ncf) die("files 4 et 59 incompatibles");
    if (!g_sym_variant) {
      double* tmp = (double*)xcalloc((size_t)ncf + 4, sizeof(double));
      for (int i = 1; i <= metat; i++) {
        int mncf = (i - 1) * ncf;
        for (int k = 1; k <= ncf; k++) tmp[iord60[k]] = c[mncf + k];
        for (int k = 1; k <= ncf; k++) c[mncf + k] = tmp[k];
      }
      free(tmp);
    }
    for (int i = 1; i <= ncf; i++) hdiag[i] = hdig(i);
    free(iord60);
  }
  if (ityper >= 0) {
    /* degen (brdnee.f:299): rotation of degenerate roots */
    if (metat > 1) {
      int jj = 0;
      for (int m = 1; m <= metat - 1; m++) {
        if (m <= jj) continue;
        jj = m - 1;
        int mn1 = m + 1;
        for (int n = mn1; n <= metat; n++) {
          jj = jj + 1;
          if (fabs(e[n] - e[m]) > 1.0e-6) break;
        }
        if (jj == m) continue;
        if (jj != mn1) {
          printf(" attention degenerescence multiple\n");
          continue;
        }
        /* brdnee.f:420-480: the first spin-flip pair whose weights differ on
           root m and whose rotation by atan(-(c11+c12)/(c21+c22)) makes
           them equal (to 1e-4) rotates roots m and m+1 */
        int mncf1 = m * ncf - ncf, mncf2 = mncf1 + ncf;
        for (int k = 1; k <= ncf; k++) {
          if (ysaut[k]) continue;
          int nespk = nesp[k];
          if (nespk == 0) continue;
          int done = 0;
          for (int ll = 1; ll <= nespk; ll++) {
            double c11 = c[mncf1 + k], c12 = c[mncf1 + k + ll];
            double c1 = fabs(c11), c2 = fabs(c12);
            if (fabs(c1 - c2) < 1.0e-5) continue;
            double c21 = c[mncf2 + k], c22 = c[mncf2 + k + ll];
            double cc = c21 + c22;
            if (fabs(cc) < 1.0e-8) continue;
            double tgphi = -(c11 + c12) / cc;
            double phi = atan(tgphi);
            double cs = cos(phi), si = sin(phi);
            c1 = c11 * cs + c21 * si;
            c2 = c12 * cs + c22 * si;
            c1 = fabs(c1);
            c2 = fabs(c2);
            double c3 = fabs(c1 - c2);
            if (c3 >= 1.0e-4) continue;
            printf(" les etats %2d et %2d sont degeneres: symmetrisation par rotation\n", m, mn1);
            for (int i = 1; i <= ncf; i++) {
              double a = c[mncf1 + i] * cs + c[mncf2 + i] * si;
              c[mncf2 + i] = -c[mncf1 + i] * si + c[mncf2 + i] * cs;
              c[mncf1 + i] = a;
            }
            done = 1;
            break;
          }
          if (done) break;
        }
      }
    }
    /* ygen: cipsym makes every determinant a generator (cipsym/ic001.f:179);
       cip keeps those with |c| >= coeff on at least one root (cip/ic001.f:751) */
    for (int k = 1; k <= ncf; k++) {
      if (g_sym_variant) {
        ygen[k] = 1;
      } else {
        for (int i = 1; i <= metat; i++)
          if (fabs(c[(i - 1) * ncf + k]) >= coeff) ygen[k] = 1;
      }
    }
  }

  for (int i = 1; i <= mnorb; i++) yoc[i] = 0;
  /* Fock operator occupations (cip.f:75-90) */
  for (int i = 1; i <= norb; i++) {
    if (tocom[i] > 1.0) {
      tocom[i + norb] = tocom[i] - 1.0;
      tocom[i] = 1.0;
    } else {
      tocom[i + norb] = 0.0;
    }
  }
  for (int i = 1; i <= noca; i++) {
    tocom[i] -= 1.0;
    tocom[i + norb] -= 1.0;
  }
  /* faifoc.f */
  for (int l = 1; l <= norb; l++) {
    double t = fdiag[l];
    int lj = num(l);
    for (int j = 1; j <= norb; j++) {
      lj = lj + 1;
      if (j > l) lj = num(j) + l;
      t = t + (tocom[j] + tocom[j + norb]) * aj[lj];
    }
    double tt = t;
    lj = num(l);
    for (int j = 1; j <= norb; j++) {
      lj = lj + 1;
      if (j > l) lj = num(j) + l;
      t = t - tocom[j] * ak[lj];
      tt = tt - tocom[j + norb] * ak[lj];
    }
    fmpb[l] = t;
    fmpb[l + norb] = tt;
  }
  for (int i = 1; i <= norb; i++) {
    fmpb[i] = (fmpb[i] + fmpb[i + norb]) * 0.5;
    fmpb[i + norb] = fmpb[i];
  }
  /* zero order (cip.f:99-135) */
  if (metat == 1) ybrd = 0;
  double* empdet = (double*)xcalloc((size_t)ncf + 4, sizeof(double));
  for (int i = 1; i <= ncf; i++) empdet[i] = hmp(i);
  for (int m = 1; m <= metat; m++) {
    e2vp[m] = 0; e2mp[m] = 0; e2b[m] = 0; emp[m] = 0; eb[m] = 0;
    double t = 0;
    int jn = (m - 1) * ncf;
    for (int i = 1; i <= ncf; i++) {
      int ij = jn + i;
      /* cip.f:113 tests ysaut through a COMMON whose layout differs from
         deter's; that view reads as .false., so every determinant counts */
      if (!(t > fabs(c[ij]))) t = fabs(c[ij]);
      emp[m] = emp[m] + c[ij] * c[ij] * empdet[i];
      eb[m] = eb[m] + (c[ij] * c[ij] * hdiag[i]);
    }
    teste[m] = test;
    taum[m] = 1.0;
    if (yselm) {
      teste[m] = t * test;
      if (ityper >= 0) taum[m] = 1.0 / t;
    }
  }
  printf(" energie de reference: %15.6f\n", escf);
  write_unit4_zero_order(n04, empdet);
  brdnee_itm();
  for (int m = 1; m <= metat; m++) {
    e2mp[m] = 0; psimp[m] = 0; psivp[m] = 0; e2vp[m] = 0; e2b[m] = 0;
  }
  ietat = 0;
  dpivot = 0.0;
  int nf = ncf + 1;
  nd[nf] = nd[ncf] + ne[ncf] + 1;
  if (nd[nf] + 32 > ntp_cap) die("internal: trou/part too small");

  ikk_buf = (int*)xcalloc((size_t)ncf + 4, sizeof(int));
  stok_buf = (double*)xcalloc((size_t)ncf + 4, sizeof(double));
  irapid = (int*)xcalloc((size_t)ncf + 4, sizeof(int));

  if (mask_path) {
    FILE* fm = fopen(mask_path, "rb");
    if (!fm) die("cannot open mask %s", mask_path);
    gen_mask = (unsigned char*)xcalloc((size_t)ncf + 4, 1);
    if (fread(gen_mask + 1, 1, (size_t)ncf, fm) != (size_t)ncf) die("short genmask");
    fclose(fm);
  }
  if (cand_path) {
    cand_log = fopen(cand_path, "wb");
    if (!cand_log) die("cannot open %s", cand_path);
  }

  /* cip.f:200-221: with ityper < 0 the determinants are ordered by
     increasing diagonal energy, the (empty) effective Hamiltonians written
     to unit 4, S written to unit 60, and the run stops (cip.f:236) */
  int* iord = (int*)xcalloc((size_t)ncf + 4, sizeof(int));
  for (int k = 1; k <= ncf; k++) iord[k] = k; /* deter.f:184 */
  if (ityper < 0) {
    double* ee = (double*)xcalloc((size_t)ncf + 4, sizeof(double));
    for (int ii = 1; ii <= ncf; ii++) ee[ii] = -hdig(ii);
    shell(ee, iord, ncf);
    free(ee);
    int nbr = metat * (metat + 1) / 2;
    double* zero = (double*)xcalloc((size_t)nbr + 2, sizeof(double));
    write_unit4_heff(n04, zero, zero, zero, zero);
    free(zero);
  }
  /* rewrite unit 60 when ymoyen: S (v=1) then the selected perturbers
     (cip.f:222-234); without ymoyen nothing is written to it */
  det_m = det_n = 0;
  det_ntot = 0;
  if (ymoyen) {
    f60 = fopen(n60, "wb");
    if (!f60) die("cannot rewrite %s", n60);
    double zero[64] = {0};
    for (int kss = 1; kss <= ncf; kss++) {
      int ks = iord[kss];
      int necst = ne[ks];
      int nts[16], nps[16];
      int necsv = necst == 0 ? 1 : necst;
      for (int ls = 1; ls <= necsv; ls++) {
        nts[ls] = trou[nd[ks] + ls];
        nps[ls] = part[nd[ks] + ls];
      }
      pie(necst, nts, nps, 1.0, zero);
    }
    fine();
  }
  free(iord);
  if (ityper < 0) {
    if (f60) fclose(f60);
    FILE* fj = fopen(json_path, "w");
    if (fj) {
      fprintf(fj, "{\n  \"ncf\": %d, \"metat\": %d, \"norb\": %d, \"noca\": %d, \"ntot60\": %lld\n}\n", ncf,
              metat, norb, noca, det_ntot);
      fclose(fj);
    }
    free(r.b);
    return 0;
  }
  /* --plan: timing of sampled generator sets on inputs read once (the
     perturbation loop only, by this process's clock) */
  long long plan_n[4096];
  double plan_t[4096];
  int nplan = 0;
  if (plan_path) {
    FILE* fp = fopen(plan_path, "r");
    if (!fp) die("cannot open plan %s", plan_path);
    if (!gen_mask) gen_mask = (unsigned char*)xcalloc((size_t)ncf + 4, 1);
    run_pertu_ref = 0;
    char line[65536];
    while (fgets(line, sizeof line, fp) && nplan < 4096) {
      char* q = line;
      char* e;
      long long m = strtoll(q, &e, 10);
      if (e == q) continue;
      q = e;
      memset(gen_mask, 0, (size_t)ncf + 4);
      for (;;) {
        long k = strtol(q, &e, 10);
        if (e == q) break;
        q = e;
        if (k >= 1 && k <= ncf) gen_mask[k] = 1;
      }
      samp_m = samp_M > 1 ? m % samp_M : 0;
      samp_seq = 0;
      const long long n0 = n_processed;
      const double ta = now_s();
      if (ypertu) pertu();
      if (ypertu) diexcit();
      plan_t[nplan] = now_s() - ta;
      plan_n[nplan++] = n_processed - n0;
    }
    fclose(fp);
  }
  double t0 = now_s();
  if (ypertu && !plan_path) pertu();
  double t1 = now_s();
  if (ypertu && !plan_path) diexcit();
  double t2 = now_s();
  if (ymoyen) {
    fine();
    fclose(f60);
  }
  if (cand_log) fclose(cand_log);

  write_unit4_results(n04);
  printf("0 ont ete generes:    %10lld  etats efficaces\n", ietat);
  printf(" la contribution du plus grand determinant non ecrit est %8.6f\n", dpivot);
  if (g_sym_variant) {
    printf("nombre de determinants sur la file 60\n");
    printf("%12lld%12d\n", det_ntot, metat);
  }
  for (int m = 1; m <= metat; m++)
    printf("  %2d  %14.8f  %14.8f  %14.8f  %14.8f\n", numero[m], e[m], e2mp[m], e2vp[m], e2b[m]);

  /* unit 33 records (stkener.f): (char*40, real*8 x(n)) without count */
  {
    FILE* f33 = fopen(n33, "ab");
    if (f33) {
      const char* names[4] = {"energies CIPSI var ", "energies CIPSI mpb ", "energies CIPSI envp",
                              "energies CIPSI enb "};
      double* vals[4] = {NULL, e2mp, e2vp, e2b};
      double etot[64];
      for (int m = 1; m <= metat; m++) etot[m] = e[m] + escf;
      vals[0] = etot;
      for (int q = 0; q < 4; q++) {
        wbuf_t w = {0};
        char typ[41];
        char tmp[128];
        snprintf(tmp, sizeof tmp, "%s%s", names[q], title);
        snprintf(typ, sizeof typ, "%-40.40s", tmp);
        wb_put(&w, typ, 40);
        for (int m = 1; m <= metat; m++) wb_r8(&w, vals[q][m]);
        wb_flush(f33, &w);
        free(w.b);
        /* stkener.f:9-12: the record's name, then its values on a line */
        printf(" *************************************\n");
        printf(" %s stockee sur la file 33\n", typ);
        for (int m = 1; m <= metat; m++) printf(" %24.16E", vals[q][m]);
        printf("\n *************************************\n");
      }
      fclose(f33);
    }
  }

  FILE* fj = fopen(json_path, "w");
  if (fj) {
    fprintf(fj, "{\n  \"ncf\": %d, \"metat\": %d, \"norb\": %d, \"noca\": %d,\n", ncf, metat, norb,
            noca);
    fprintf(fj, "  \"ietat\": %lld, \"n_processed\": %lld, \"ntot60\": %lld,\n", ietat, n_processed,
            det_ntot);
    fprintf(fj, "  \"dpivot\": %.17g,\n", dpivot);
    double cm[64], cv[64], cb[64];
    for (int m = 1; m <= metat; m++) {
      cm[m] = ks_mp[m] + kc_mp[m];
      cv[m] = ks_vp[m] + kc_vp[m];
      cb[m] = ks_b[m] + kc_b[m];
    }
    const char* nm[11] = {"e2mp", "e2vp", "e2b", "psimp", "psivp", "cond_e2mp", "cond_e2vp", "cond_e2b",
                          "comp_e2mp", "comp_e2vp", "comp_e2b"};
    double* ar[11] = {e2mp, e2vp, e2b, psimp, psivp, cond_mp, cond_vp, cond_b, cm, cv, cb};
    for (int q = 0; q < 11; q++) {
      fprintf(fj, "  \"%s\": [", nm[q]);
      for (int m = 1; m <= metat; m++) fprintf(fj, "%s%.17g", m > 1 ? ", " : "", ar[q][m]);
      fprintf(fj, "],\n");
    }
    fprintf(fj, "  \"e\": [");
    for (int m = 1; m <= metat; m++) fprintf(fj, "%s%.17g", m > 1 ? ", " : "", e[m]);
    fprintf(fj, "],\n  \"emp\": [");
    for (int m = 1; m <= metat; m++) fprintf(fj, "%s%.17g", m > 1 ? ", " : "", emp[m]);
    fprintf(fj, "],\n  \"eb\": [");
    for (int m = 1; m <= metat; m++) fprintf(fj, "%s%.17g", m > 1 ? ", " : "", eb[m]);
    fprintf(fj, "],\n  \"nom\": [");
    for (int i = 1; i <= nclass; i++) fprintf(fj, "%s%lld", i > 1 ? ", " : "", nom[i]);
    fprintf(fj, "],\n  \"nam\": [");
    for (int m = 1; m <= metat; m++) {
      fprintf(fj, "%s[", m > 1 ? ", " : "");
      for (int i = 1; i <= nclass; i++) fprintf(fj, "%s%lld", i > 1 ? ", " : "", nam[i][m]);
      fprintf(fj, "]");
    }
    fprintf(fj, "],\n  \"tabmp\": [");
    for (int m = 1; m <= metat; m++) {
      fprintf(fj, "%s[", m > 1 ? ", " : "");
      for (int i = 1; i <= nclass; i++) fprintf(fj, "%s%.17g", i > 1 ? ", " : "", tabmp[i][m]);
      fprintf(fj, "]");
    }
    fprintf(fj, "],\n  \"tabvp\": [");
    for (int m = 1; m <= metat; m++) {
      fprintf(fj, "%s[", m > 1 ? ", " : "");
      for (int i = 1; i <= nclass; i++) fprintf(fj, "%s%.17g", i > 1 ? ", " : "", tabvp[i][m]);
      fprintf(fj, "]");
    }
    fprintf(fj, "],\n  \"plan\": [");
    for (int i = 0; i < nplan; i++) fprintf(fj, "%s[%lld, %.6f]", i ? ", " : "", plan_n[i], plan_t[i]);
    fprintf(fj, "],\n  \"t_pertu_s\": %.6f, \"t_diexcit_s\": %.6f\n}\n", t1 - t0, t2 - t1);
    fclose(fj);
  }
  free(r.b);
  return 0;
}
