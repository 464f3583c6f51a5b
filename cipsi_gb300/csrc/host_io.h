// host_io.h -- what the drop-in executables read and write as the Fortran
// reference does: sequential unformatted records (a 4-byte length before
// and after each record), namelist groups on standard input, and unit file
// names built from a namelist (nomf.f / nomfil.f).  Shared by the cip/cipsym
// drop-in (cip_host.cpp) and the moy drop-in (moy_host.cpp).
#pragma once

#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace cipsi_host {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ------------------------------------------------ Fortran sequential files
struct Record {
  std::vector<unsigned char> b;
  size_t pos = 0;
  template <typename T>
  T get() {
    if (pos + sizeof(T) > b.size()) throw Error("record too short");
    T v;
    std::memcpy(&v, b.data() + pos, sizeof(T));
    pos += sizeof(T);
    return v;
  }
};

inline std::vector<Record> read_records(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error("cannot open " + path);
  std::vector<Record> out;
  for (;;) {
    int32_t n1;
    if (!f.read(reinterpret_cast<char*>(&n1), 4)) break;
    if (n1 < 0) throw Error("bad record length in " + path);
    Record r;
    r.b.resize((size_t)n1);
    if (n1 && !f.read(reinterpret_cast<char*>(r.b.data()), n1)) throw Error("truncated record in " + path);
    int32_t n2;
    if (!f.read(reinterpret_cast<char*>(&n2), 4) || n2 != n1) throw Error("bad record marker in " + path);
    out.push_back(std::move(r));
  }
  return out;
}

struct RecWriter {
  std::vector<unsigned char> b;
  template <typename T>
  void put(T v) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&v);
    b.insert(b.end(), p, p + sizeof(T));
  }
  void put_bytes(const char* s, size_t n) { b.insert(b.end(), s, s + n); }
  void flush(std::FILE* f) {
    const int32_t n = (int32_t)b.size();
    std::fwrite(&n, 4, 1, f);
    if (n) std::fwrite(b.data(), 1, b.size(), f);
    std::fwrite(&n, 4, 1, f);
    b.clear();
  }
};

// ---------------------------------------------------------------- namelists
// A namelist group read as the Fortran runtime reads it: from "&group" to
// "&end" or "/"; "name = values" with names in any case; values separated by
// commas and/or blanks; "r*c" for r copies of c; "r*", or nothing between
// two commas, for null values (the element keeps its value); "name(i) =
// values" assigning from element i on; "!" starting a comment to the end of
// the line.  Each name maps to the elements assigned (1-based index -> text).
struct Namelist {
  std::map<std::string, std::map<int, std::string>> kv;
  std::map<std::string, int> last;  // the highest element a value (or a null) went to
  bool found = false;
  std::string group;
  bool has(const std::string& k) const { return kv.count(k) != 0; }
  // the value of a scalar variable, or nullptr when not assigned
  const std::string* scalar(const std::string& k) const {
    auto it = kv.find(k);
    if (it == kv.end()) return nullptr;
    if (last.at(k) > 1) throw Error("erreur dans la namelist " + group + ": too many values for " + k);
    auto e = it->second.find(1);
    return e == it->second.end() ? nullptr : &e->second;
  }
  // the elements assigned to an array variable of `bound` elements
  const std::map<int, std::string>& array(const std::string& k, int bound) const {
    static const std::map<int, std::string> none;
    auto it = kv.find(k);
    if (it == kv.end()) return none;
    if (last.at(k) > bound)
      throw Error("erreur dans la namelist " + group + ": " + k + " has more than " + std::to_string(bound) +
                  " elements");
    return it->second;
  }
};

inline std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

inline Namelist parse_namelist(const std::string& text, const std::string& group,
                        const std::set<std::string>& names) {
  Namelist nl;
  nl.group = group;
  const std::string lt = lower(text), key = "&" + lower(group);
  size_t pos = std::string::npos;
  for (size_t p = lt.find(key); p != std::string::npos; p = lt.find(key, p + 1)) {
    const char nx = p + key.size() < lt.size() ? lt[p + key.size()] : ' ';
    if (!std::isalnum((unsigned char)nx) && nx != '_') {
      pos = p + key.size();
      break;
    }
  }
  if (pos == std::string::npos) return nl;
  nl.found = true;
  auto bad = [&](const std::string& m) { throw Error("erreur dans la namelist " + group + ": " + m); };
  std::string cur;
  int idx = 1;
  bool need_sep = false;  // a value was just read: the next comma only separates
  size_t i = pos;
  const size_t n = text.size();
  auto put = [&](const std::string& v) {
    if (cur.empty()) bad("value without a name");
    if (!v.empty()) nl.kv[cur][idx] = v;  // a null leaves the element as it is
    nl.last[cur] = std::max(nl.last[cur], idx);
    ++idx;
  };
  while (i < n) {
    const char ch = text[i];
    if (std::isspace((unsigned char)ch)) {
      ++i;
      continue;
    }
    if (ch == '!') {
      while (i < n && text[i] != '\n') ++i;
      continue;
    }
    if (ch == '/' || ch == '&') break;
    if (ch == ',') {
      if (!need_sep && !cur.empty()) {  // null value
        nl.last[cur] = std::max(nl.last[cur], idx);
        ++idx;
      }
      need_sep = false;
      ++i;
      continue;
    }
    std::string tok;
    bool quoted = false;
    if (ch == '\'' || ch == '"') {
      quoted = true;
      const char q = text[i++];
      for (; i < n; ++i) {
        if (text[i] == q) {
          if (i + 1 < n && text[i + 1] == q) {  // doubled quote
            tok += q;
            ++i;
            continue;
          }
          ++i;
          break;
        }
        tok += text[i];
      }
    } else {
      while (i < n && !std::isspace((unsigned char)text[i]) && text[i] != ',' && text[i] != '=' &&
             text[i] != '/' && text[i] != '!')
        tok += text[i++];
    }
    size_t r = i;
    while (r < n && std::isspace((unsigned char)text[r])) ++r;
    if (!quoted && r < n && text[r] == '=') {
      std::string name = lower(tok);
      idx = 1;
      if (const size_t lp = name.find('('); lp != std::string::npos) {
        if (name.back() != ')') bad("bad subscript in " + tok);
        idx = std::atoi(name.c_str() + lp + 1);
        name = name.substr(0, lp);
        if (idx < 1) bad("bad subscript in " + tok);
      }
      if (!names.count(name)) bad("unknown name " + name);
      cur = name;
      nl.kv[cur];
      nl.last[cur];
      need_sep = false;
      i = r + 1;
      continue;
    }
    const size_t star = quoted ? std::string::npos : tok.find('*');
    if (star != std::string::npos && star > 0 &&
        tok.find_first_not_of("0123456789") == star) {  // r*c or r*
      const int rep = std::atoi(tok.substr(0, star).c_str());
      std::string c = tok.substr(star + 1);
      if (c.size() >= 2 && (c[0] == '\'' || c[0] == '"') && c.back() == c[0]) c = c.substr(1, c.size() - 2);
      for (int q = 0; q < rep; ++q) put(c);
    } else {
      if (quoted && tok.empty()) tok = " ";  // an empty string is a value, not a null
      put(tok);
    }
    need_sep = true;
  }
  return nl;
}

inline double to_real(std::string s) {
  for (auto& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  size_t used = 0;
  const double v = std::stod(s, &used);
  if (used != s.size()) throw Error("erreur dans la namelist: bad real value " + s);
  return v;
}
inline int to_int(const std::string& s) {
  size_t used = 0;
  const int v = std::stoi(s, &used);
  if (used != s.size()) throw Error("erreur dans la namelist: bad integer value " + s);
  return v;
}
inline bool to_logical(const std::string& s) {
  size_t i = 0;
  while (i < s.size() && s[i] == '.') ++i;
  if (i >= s.size() || !std::strchr("tTfF", s[i]))
    throw Error("erreur dans la namelist: bad logical value " + s);
  return s[i] == 't' || s[i] == 'T';
}

// nomf.f: a unit's file name is the prefix up to its first blank followed
// by the root name (10 characters) up to its first blank -- nothing of the
// root when its 10 characters hold no blank; a non-blank name1 (90
// characters) replaces both (nomfil.f)
inline std::string unit_file(const Namelist& cf, const char* root_key, const char* name1_key, const char* root_default,
                      const std::string& dir) {
  std::string f;
  if (const std::string* v = cf.scalar(name1_key); v && v->find_first_not_of(' ') != std::string::npos) {
    f = v->substr(0, 90);
    while (!f.empty() && f.back() == ' ') f.pop_back();
  } else {
    std::string prefix, root = root_default;
    if (const std::string* p = cf.scalar("prefix")) prefix = p->substr(0, 80);
    prefix = prefix.substr(0, prefix.find(' '));
    if (const std::string* r = cf.scalar(root_key)) root = *r;
    root.resize(10, ' ');
    const size_t b = root.find(' ');
    f = prefix + (b == std::string::npos ? std::string() : root.substr(0, b));
  }
  if (!f.empty() && f[0] != '/') f = dir + "/" + f;
  return f;
}

}  // namespace cipsi_host
