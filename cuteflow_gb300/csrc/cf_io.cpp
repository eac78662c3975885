/*
 * cf_io.cpp -- the reference's input files behind the C ABI, so that a CuteFlow case
 * directory runs unchanged:
 *
 *   donnees.f     the donnees_namelist (lec_donnees, maillage.cuf:168-193; the namelist
 *                 global_data.cuf:65-94), Fortran namelist syntax;
 *   mesh file     the ASCII triangle mesh (lec_mail_tri, maillage.cuf:196-313), Fortran
 *                 list-directed records;
 *   fich_sol_init the element initial condition (read_initial_condition,
 *                 initial_condition.cuf:82-102), and the same layout written back
 *                 (save_sol_for_restart, pre_post_traitement.cuf:498-512).
 *
 *   CGNS mesh     is_cgns = 1 (lec_mail_cgns, maillage.cuf:398-778), read by cf_cgns.cpp from the
 *                 HDF5 container directly (no libcgns).
 * Host code only; nothing here touches the GPU.
 */
#include <cctype>
#include <climits>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <new>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cf_internal.h"

struct cf_case {
  /* storage behind the cf_mesh pointers */
  std::vector<double> x, y, z, manning_nd, manning_elt;
  std::vector<int32_t> tri, ndinput, numero_ndinput, ndoutput, numero_ndoutput, ndwall;
  cf_mesh mesh{};
  cf_params params{};
  cf_ic ic{};
  double ts = 0.0;
  int32_t solinit = 0;
  int32_t is_cgns = 0;
  std::vector<double> U0;  /* solinit = 1: the state of fich_sol_init */
  double tc_init = 0.0;    /* the first value of fich_sol_init (read, not used: main.cuf:182) */
  std::string meshfile_path = "./", meshfile, fich_sol_init;
  std::vector<std::string> inlet_name, outlet_name;   /* CGNS boundary names of the inlets / outlets */
};

namespace {

thread_local std::string g_io_error;

int io_fail(int code, const std::string& msg) {
  g_io_error = msg;
  return code;
}

std::string lower(std::string s) {
  for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

/* A Fortran real or integer constant: d/D exponents as e (1.0d-5), no trailing junk. */
bool parse_real(const std::string& tok, double& out) {
  std::string t = tok;
  for (char& ch : t)
    if (ch == 'd' || ch == 'D') ch = 'e';
  if (t.empty()) return false;
  char* end = nullptr;
  errno = 0;
  out = std::strtod(t.c_str(), &end);
  return end && *end == '\0' && errno != ERANGE;
}

bool parse_int(const std::string& tok, int64_t& out) {
  if (tok.empty()) return false;
  char* end = nullptr;
  errno = 0;
  long long v = std::strtoll(tok.c_str(), &end, 10);
  if (!end || *end != '\0' || errno == ERANGE) return false;
  out = v;
  return true;
}

/* ---- list-directed records ------------------------------------------------------------- */

/* Fortran list-directed READ: every statement starts at the next record and reads as many
 * records as its items need; the rest of its last record is skipped.  Values are separated by
 * blanks or commas; r*c repeats c r times; a slash ends the statement's input. */
class ListReader {
 public:
  explicit ListReader(std::istream& in) : in_(in) {}

  /* the next READ of n items into toks (false at end of file before n items) */
  bool read(size_t n, std::vector<std::string>& toks) {
    toks.clear();
    std::string line;
    while (toks.size() < n) {
      if (!std::getline(in_, line)) return false;
      ++lineno_;
      if (split(line, n, toks)) break;   /* slash */
    }
    return toks.size() >= n;
  }
  /* a READ of one character item (the section titles): consumes one record */
  bool skip_title() {
    std::string line;
    while (std::getline(in_, line)) {
      ++lineno_;
      for (char ch : line)
        if (!std::isspace((unsigned char)ch)) return true;
    }
    return false;
  }
  long line() const { return lineno_; }

 private:
  static bool split(const std::string& line, size_t n, std::vector<std::string>& toks) {
    size_t i = 0;
    while (i < line.size() && toks.size() < n) {
      const char ch = line[i];
      if (std::isspace((unsigned char)ch) || ch == ',') { ++i; continue; }
      if (ch == '/') return true;
      size_t j = i;
      while (j < line.size() && !std::isspace((unsigned char)line[j]) && line[j] != ',' && line[j] != '/') ++j;
      std::string tok = line.substr(i, j - i);
      const size_t star = tok.find('*');
      int64_t r = 0;
      if (star != std::string::npos && parse_int(tok.substr(0, star), r) && r > 0) {
        const std::string c = tok.substr(star + 1);
        for (int64_t k = 0; k < r; ++k) toks.push_back(c);
      } else {
        toks.push_back(tok);
      }
      i = j;
    }
    return false;
  }
  std::istream& in_;
  long lineno_ = 0;
};

/* ---- the namelist ----------------------------------------------------------------------- */

struct NmlValue {
  std::vector<std::string> items;  /* raw values (strings unquoted) */
  int64_t index = 1;               /* first array index (name(i) = ...) */
};

/* Parse &name ... / : returns the assignments in order (names lower case). */
int parse_namelist(const std::string& text, const std::string& group,
                   std::vector<std::pair<std::string, NmlValue>>& out) {
  /* strip comments (outside quotes) */
  std::string s;
  s.reserve(text.size());
  {
    char q = 0;
    for (size_t i = 0; i < text.size(); ++i) {
      const char ch = text[i];
      if (q) {
        s += ch;
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
        s += ch;
      } else if (ch == '!') {
        while (i < text.size() && text[i] != '\n') ++i;
        s += '\n';
      } else {
        s += ch;
      }
    }
  }
  const std::string ls = lower(s);
  const size_t start = ls.find("&" + lower(group));
  if (start == std::string::npos) return io_fail(CF_EINVAL, "namelist group &" + group + " not found");
  size_t i = start + 1 + group.size();
  /* tokens: names, '=', values, up to the closing slash */
  std::vector<std::string> toks;
  std::vector<bool> quoted;
  bool closed = false;
  while (i < s.size()) {
    const char ch = s[i];
    if (std::isspace((unsigned char)ch) || ch == ',') { ++i; continue; }
    if (ch == '/') { closed = true; break; }
    if (ch == '&') {  /* "&end" also closes a group */
      closed = true;
      break;
    }
    if (ch == '=') { toks.push_back("="); quoted.push_back(false); ++i; continue; }
    if (ch == '\'' || ch == '"') {
      size_t j = i + 1;
      std::string v;
      while (j < s.size()) {
        if (s[j] == ch) {
          if (j + 1 < s.size() && s[j + 1] == ch) { v += ch; j += 2; continue; }  /* doubled quote */
          break;
        }
        v += s[j++];
      }
      if (j >= s.size()) return io_fail(CF_EINVAL, "unterminated string in the namelist");
      toks.push_back(v);
      quoted.push_back(true);
      i = j + 1;
      continue;
    }
    size_t j = i;
    while (j < s.size() && !std::isspace((unsigned char)s[j]) && s[j] != ',' && s[j] != '=' && s[j] != '/' &&
           s[j] != '\'' && s[j] != '"')
      ++j;
    toks.push_back(s.substr(i, j - i));
    quoted.push_back(false);
    i = j;
  }
  if (!closed) return io_fail(CF_EINVAL, "namelist group &" + group + " is not closed by '/'");
  /* name = v1 v2 ... name = ... */
  size_t k = 0;
  while (k < toks.size()) {
    if (quoted[k] || k + 1 >= toks.size() || toks[k + 1] != "=")
      return io_fail(CF_EINVAL, "namelist: expected 'name =' near '" + toks[k] + "'");
    std::string name = lower(toks[k]);
    NmlValue v;
    const size_t par = name.find('(');
    if (par != std::string::npos) {
      const size_t cl = name.find(')', par);
      int64_t idx = 0;
      if (cl == std::string::npos || !parse_int(name.substr(par + 1, cl - par - 1), idx) || idx < 1)
        return io_fail(CF_EINVAL, "namelist: bad array element '" + toks[k] + "'");
      v.index = idx;
      name = name.substr(0, par);
    }
    k += 2;
    while (k < toks.size() && !(k + 1 < toks.size() && !quoted[k] && toks[k + 1] == "=")) {
      const std::string& t = toks[k];
      const size_t star = quoted[k] ? std::string::npos : t.find('*');
      int64_t r = 0;
      if (star != std::string::npos && parse_int(t.substr(0, star), r) && r > 0) {
        for (int64_t q = 0; q < r; ++q) v.items.push_back(t.substr(star + 1));
      } else {
        v.items.push_back(t);
      }
      ++k;
    }
    out.emplace_back(name, v);
  }
  return CF_OK;
}

/* The keys of donnees_namelist (global_data.cuf:65-94). */
const char* const kKnownKeys[] = {
    "gp", "is_override_manning", "override_manning", "is_cgns", "meshfile_path", "meshfile", "elt_bound",
    "nombre_entrees", "nombre_sorties", "eqlin_barrage", "x1eqbar", "x2eqbar", "y1eqbar", "y2eqbar", "h_amont",
    "u_amont", "v_amont", "h_aval", "u_aval", "v_aval", "plan", "xplan", "yplan", "zplan", "xpoint", "ypoint",
    "zpoint", "solinit", "fich_sol_init", "inlet", "inlet_name", "debitglob", "debit_var", "loi_debitglob",
    "outlet", "outlet_name", "h_sortie", "iflux", "ilimiteur", "iupwind", "tolisec", "friction", "fricimplic",
    "diffusion", "ts", "cfl", "tol_reg_perm", "is_dt_constant", "constant_dt", "freqaffich", "tolaffiche",
    "sol_z_offset", "solrestart", "solvisu", "visu_snapshots", "sortie_finale_bluekenue"};

int apply_namelist(const std::vector<std::pair<std::string, NmlValue>>& nml, cf_case& C) {
  cf_params& p = C.params;
  cf_ic& ic = C.ic;
  for (const auto& kv : nml) {
    const std::string& k = kv.first;
    const NmlValue& v = kv.second;
    bool known = false;
    for (const char* kk : kKnownKeys) known |= (k == kk);
    if (!known) return io_fail(CF_EINVAL, "namelist: unknown key '" + k + "' (not in donnees_namelist)");
    if (v.items.empty()) continue;  /* a null value leaves the variable unchanged */
    auto real1 = [&](double& dst) -> int {
      double d;
      if (!parse_real(v.items[0], d)) return io_fail(CF_EINVAL, "namelist: bad real for '" + k + "'");
      dst = d;
      return CF_OK;
    };
    auto int1 = [&](int32_t& dst) -> int {
      int64_t d;
      if (!parse_int(v.items[0], d)) return io_fail(CF_EINVAL, "namelist: bad integer for '" + k + "'");
      dst = (int32_t)d;
      return CF_OK;
    };
    auto realv = [&](double* arr) -> int {
      for (size_t i = 0; i < v.items.size(); ++i) {
        const int64_t at = v.index - 1 + (int64_t)i;
        if (at >= CF_MAX_IO) return io_fail(CF_EINVAL, "namelist: '" + k + "' has more than 20 values");
        double d;
        if (!parse_real(v.items[i], d)) return io_fail(CF_EINVAL, "namelist: bad real for '" + k + "'");
        arr[at] = d;
      }
      return CF_OK;
    };
    int rc = CF_OK;
    int32_t tmp = 0;
    if (k == "gp") rc = real1(p.gp);
    else if (k == "is_override_manning") rc = int1(p.is_override_manning);
    else if (k == "override_manning") rc = real1(p.override_manning);
    else if (k == "is_cgns") rc = int1(C.is_cgns);
    else if (k == "meshfile_path") C.meshfile_path = v.items[0];
    else if (k == "meshfile") C.meshfile = v.items[0];
    else if (k == "inlet_name" || k == "outlet_name") {
      auto& names = (k == "inlet_name") ? C.inlet_name : C.outlet_name;
      for (size_t i = 0; i < v.items.size(); ++i) {
        const int64_t at = v.index - 1 + (int64_t)i;
        if (at < 0 || at >= CF_MAX_IO) return io_fail(CF_EINVAL, "namelist: '" + k + "' has more than 20 values");
        if ((int64_t)names.size() <= at) names.resize((size_t)at + 1);
        names[(size_t)at] = v.items[i];
      }
    }
    else if (k == "nombre_entrees") rc = int1(C.mesh.nombre_entrees);
    else if (k == "nombre_sorties") rc = int1(C.mesh.nombre_sorties);
    else if (k == "eqlin_barrage") rc = int1(ic.eqlin_barrage);
    else if (k == "x1eqbar") rc = real1(ic.x1eqbar);
    else if (k == "x2eqbar") rc = real1(ic.x2eqbar);
    else if (k == "y1eqbar") rc = real1(ic.y1eqbar);
    else if (k == "y2eqbar") rc = real1(ic.y2eqbar);
    else if (k == "h_amont") rc = real1(ic.h_amont);
    else if (k == "u_amont") rc = real1(ic.u_amont);
    else if (k == "v_amont") rc = real1(ic.v_amont);
    else if (k == "h_aval") rc = real1(ic.h_aval);
    else if (k == "u_aval") rc = real1(ic.u_aval);
    else if (k == "v_aval") rc = real1(ic.v_aval);
    else if (k == "plan") rc = int1(ic.plan);
    else if (k == "xplan") rc = real1(ic.xplan);
    else if (k == "yplan") rc = real1(ic.yplan);
    else if (k == "zplan") rc = real1(ic.zplan);
    else if (k == "xpoint") rc = real1(ic.xpoint);
    else if (k == "ypoint") rc = real1(ic.ypoint);
    else if (k == "zpoint") rc = real1(ic.zpoint);
    else if (k == "solinit") rc = int1(C.solinit);
    else if (k == "fich_sol_init") C.fich_sol_init = v.items[0];
    else if (k == "inlet") {
      /* data_transfer.cuf:43-55 */
      std::string t = lower(v.items[0]);
      t.erase(0, t.find_first_not_of(' '));
      t.erase(t.find_last_not_of(' ') + 1);
      if (t == "transm") p.inlet = 1;
      else if (t == "inflow") p.inlet = 2;
      else if (t == "phys_inflow") p.inlet = 3;
      else return io_fail(CF_EINVAL, "namelist: bad inlet '" + v.items[0] + "'");
    } else if (k == "outlet") {
      std::string t = lower(v.items[0]);
      t.erase(0, t.find_first_not_of(' '));
      t.erase(t.find_last_not_of(' ') + 1);
      if (t == "fixedheight") p.outlet = 1;
      else if (t == "transm") p.outlet = 2;
      else return io_fail(CF_EINVAL, "namelist: bad outlet '" + v.items[0] + "'");
    } else if (k == "debitglob") rc = realv(p.debitglob);
    else if (k == "h_sortie") rc = realv(p.h_sortie);
    else if (k == "iflux") rc = int1(p.iflux);
    else if (k == "ilimiteur") rc = int1(p.ilimiteur);
    else if (k == "tolisec") rc = real1(p.tolisec);
    else if (k == "friction") rc = int1(p.friction);
    else if (k == "fricimplic") rc = int1(p.fricimplic);
    else if (k == "ts") rc = real1(C.ts);
    else if (k == "cfl") rc = real1(p.cfl);
    else if (k == "tol_reg_perm") rc = real1(p.tol_reg_perm);
    else if (k == "is_dt_constant") rc = int1(p.is_dt_constant);
    else if (k == "constant_dt") rc = real1(p.constant_dt);
    else if (k == "diffusion") {
      rc = int1(tmp);
      if (rc == CF_OK && tmp != 0) return io_fail(CF_ENOTSUP, "namelist: diffusion is not supported by the step");
    }
    /* the remaining keys select output, naming or the CGNS path and do not affect the step */
    if (rc != CF_OK) return rc;
  }
  return CF_OK;
}

std::string join_path(const std::string& dir, const std::string& f) {
  if (f.empty() || f[0] == '/' || dir.empty()) return f;
  return dir.back() == '/' ? dir + f : dir + "/" + f;
}

std::string trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  return s.substr(a, s.find_last_not_of(" \t\r\n") - a + 1);
}

/* lec_mail_tri (maillage.cuf:196-313), one process */
int read_mesh(const std::string& path, cf_case& C) {
  std::ifstream f(path);
  if (!f) return io_fail(CF_EINVAL, "cannot open the mesh file " + path);
  ListReader r(f);
  std::vector<std::string> t;
  auto bad = [&](const char* what) {
    return io_fail(CF_EINVAL, std::string("mesh file ") + path + ", line " + std::to_string(r.line()) + ": " + what);
  };
  int64_t v = 0;
  if (!r.skip_title()) return bad("missing the node table title");
  if (!r.read(1, t) || !parse_int(t[0], v) || v < 1 || v > INT32_MAX) return bad("bad node count");
  const int64_t nnt = v;
  C.x.resize(nnt); C.y.resize(nnt); C.z.resize(nnt); C.manning_nd.resize(nnt);
  for (int64_t i = 0; i < nnt; ++i) {
    double a, b, c, d;
    if (!r.read(5, t) || !parse_real(t[1], a) || !parse_real(t[2], b) || !parse_real(t[3], c) || !parse_real(t[4], d))
      return bad("bad node record (n, x, y, z, manning)");
    C.x[i] = a; C.y[i] = b; C.z[i] = c; C.manning_nd[i] = d;
  }
  if (!r.skip_title()) return bad("missing the connectivity title");
  if (!r.read(1, t) || !parse_int(t[0], v) || v < 1 || v > INT32_MAX / 3) return bad("bad element count");
  const int64_t nelt = v;
  C.tri.resize(3 * nelt);
  C.manning_elt.resize(nelt);
  for (int64_t i = 0; i < nelt; ++i) {
    int64_t a, b, c;
    double d;
    if (!r.read(5, t) || !parse_int(t[1], a) || !parse_int(t[2], b) || !parse_int(t[3], c) || !parse_real(t[4], d))
      return bad("bad element record (n, n1, n2, n3, manning)");
    if (a < 1 || a > nnt || b < 1 || b > nnt || c < 1 || c > nnt) return bad("element node id out of range");
    C.tri[3 * i] = (int32_t)a; C.tri[3 * i + 1] = (int32_t)b; C.tri[3 * i + 2] = (int32_t)c;
    C.manning_elt[i] = d;
  }
  /* inflow and outflow nodes: with one inlet (outlet) the count alone and one node per record,
   * otherwise the count and the number of inlets, then (node, inlet number) records */
  auto io_table = [&](int32_t& nbr, std::vector<int32_t>& nodes, std::vector<int32_t>& numero) -> int {
    if (!r.skip_title()) return bad("missing an inflow/outflow title");
    int64_t n = 0, nb = 0;
    const bool numbered = nbr != 1;   /* the namelist's count selects the layout */
    if (!numbered) {
      if (!r.read(1, t) || !parse_int(t[0], n) || n < 0 || n > INT32_MAX) return bad("bad inflow/outflow node count");
    } else {
      if (!r.read(2, t) || !parse_int(t[0], n) || !parse_int(t[1], nb) || n < 0 || n > INT32_MAX || nb < 0 ||
          nb > CF_MAX_IO)
        return bad("bad inflow/outflow counts");
      nbr = (int32_t)nb;
    }
    nodes.resize(n);
    numero.resize(n);
    for (int64_t i = 0; i < n; ++i) {
      int64_t a = 0, b = 1;
      if (!r.read(numbered ? 2 : 1, t) || !parse_int(t[0], a) || (numbered && !parse_int(t[1], b)))
        return bad("bad inflow/outflow node record");
      if (a < 1 || a > nnt) return bad("inflow/outflow node id out of range");
      nodes[i] = (int32_t)a;
      numero[i] = (int32_t)b;
    }
    return CF_OK;
  };
  int rc;
  if ((rc = io_table(C.mesh.nombre_entrees, C.ndinput, C.numero_ndinput))) return rc;
  if ((rc = io_table(C.mesh.nombre_sorties, C.ndoutput, C.numero_ndoutput))) return rc;
  if (!r.skip_title()) return bad("missing the wall title");
  if (!r.read(1, t) || !parse_int(t[0], v) || v < 0 || v > INT32_MAX) return bad("bad wall node count");
  C.ndwall.resize(v);
  for (int64_t i = 0; i < v; ++i) {
    int64_t a;
    if (!r.read(1, t) || !parse_int(t[0], a) || a < 1 || a > nnt) return bad("bad wall node record");
    C.ndwall[i] = (int32_t)a;
  }
  return CF_OK;
}

/* lec_mail_cgns (maillage.cuf:398-778), one process: the mesh, its inflow/outflow node lists and
 * its per-element Manning n (unless is_override_manning, which the step applies itself); no wall
 * nodes are listed (every unmatched boundary edge is a wall, maillage.cuf:1454-1471). */
int read_cgns(const std::string& path, cf_case& C) {
  cf::CgnsMesh M;
  std::string err;
  const bool want_manning = C.params.is_override_manning != 1;
  const int rc = cf::read_cgns_mesh(path, C.inlet_name, C.outlet_name, want_manning, M, err);
  if (rc != CF_OK) return io_fail(rc, "CGNS mesh " + path + ": " + err);
  if (want_manning && !M.has_manning)
    return io_fail(CF_EINVAL, "CGNS mesh " + path + " has no Manning user data and is_override_manning = 0");
  if (!M.ndinput.empty() && C.mesh.nombre_entrees < 1)
    return io_fail(CF_EINVAL, "CGNS mesh " + path + " has inflow nodes but nombre_entrees = 0");
  if (!M.ndoutput.empty() && C.mesh.nombre_sorties < 1)
    return io_fail(CF_EINVAL, "CGNS mesh " + path + " has outflow nodes but nombre_sorties = 0");
  C.x = std::move(M.x);
  C.y = std::move(M.y);
  C.z = std::move(M.z);
  C.manning_nd.assign(C.x.size(), 0.0);
  C.tri = std::move(M.tri);
  C.manning_elt = want_manning ? std::move(M.manning_elt) : std::vector<double>(C.tri.size() / 3, C.params.override_manning);
  C.ndinput = std::move(M.ndinput);
  C.numero_ndinput = std::move(M.numero_ndinput);
  C.ndoutput = std::move(M.ndoutput);
  C.numero_ndoutput = std::move(M.numero_ndoutput);
  C.ndwall.clear();
  return CF_OK;
}

/* read_initial_condition (initial_condition.cuf:82-102) */
int read_state_file(const std::string& path, int64_t nelt, std::vector<double>& U, double& t0) {
  std::ifstream f(path);
  if (!f) return io_fail(CF_EINVAL, "cannot open the initial condition file " + path);
  ListReader r(f);
  std::vector<std::string> t;
  if (!r.read(1, t) || !parse_real(t[0], t0)) return io_fail(CF_EINVAL, path + ": bad first record (time)");
  U.resize(3 * nelt);
  for (int64_t i = 0; i < nelt; ++i) {
    if (!r.read(3, t) || !parse_real(t[0], U[3 * i]) || !parse_real(t[1], U[3 * i + 1]) ||
        !parse_real(t[2], U[3 * i + 2]))
      return io_fail(CF_EINVAL, path + ": bad record for element " + std::to_string(i + 1));
  }
  return CF_OK;
}

void fill_mesh(cf_case& C) {
  cf_mesh& m = C.mesh;
  m.nnt = (int32_t)C.x.size();
  m.nelt = (int32_t)C.manning_elt.size();
  m.x = C.x.data();
  m.y = C.y.data();
  m.z = C.z.data();
  m.tri = C.tri.data();
  m.manning_elt = C.manning_elt.data();
  m.ndinput = C.ndinput.data();
  m.numero_ndinput = C.numero_ndinput.data();
  m.ndoutput = C.ndoutput.data();
  m.numero_ndoutput = C.numero_ndoutput.data();
  m.ndwall = C.ndwall.data();
  m.ndi = (int32_t)C.ndinput.size();
  m.ndo = (int32_t)C.ndoutput.size();
  m.ndw = (int32_t)C.ndwall.size();
}

}  // namespace

extern "C" {

static int case_read_impl(const char* dir, const char* namelist_file, cf_case** out);

int cf_case_read(const char* dir, const char* namelist_file, cf_case** out) {
  /* no C++ exception crosses the C ABI: a file whose counts outrun host memory is an error */
  try {
    return case_read_impl(dir, namelist_file, out);
  } catch (const std::bad_alloc&) {
    if (out) *out = nullptr;
    return io_fail(CF_ENOMEM, "host allocation failed reading the case (counts in the files too large?)");
  } catch (const std::length_error&) {
    if (out) *out = nullptr;
    return io_fail(CF_EINVAL, "counts in the case files too large");
  }
}

static int case_read_impl(const char* dir, const char* namelist_file, cf_case** out) {
  if (!out) return io_fail(CF_EINVAL, "out is NULL");
  *out = nullptr;
  const std::string d = dir ? dir : ".";
  const std::string nml_path = join_path(d, namelist_file ? namelist_file : "donnees.f");
  std::ifstream f(nml_path);
  if (!f) return io_fail(CF_EINVAL, "cannot open the namelist file " + nml_path);
  std::stringstream ss;
  ss << f.rdbuf();
  std::unique_ptr<cf_case> C(new (std::nothrow) cf_case());
  if (!C) return io_fail(CF_ENOMEM, "host allocation failed");
  cf_default_params(&C->params);
  C->params.friction = 0;          /* friction=0 is the namelist's initial value (global_data.cuf:31) */
  C->mesh.nombre_entrees = 1;
  C->mesh.nombre_sorties = 1;
  std::vector<std::pair<std::string, NmlValue>> nml;
  int rc = parse_namelist(ss.str(), "donnees_namelist", nml);
  if (rc == CF_OK) rc = apply_namelist(nml, *C);
  if (rc == CF_OK) {
    /* trim(adjustl(meshfile_path)) // trim(adjustl(meshfile)), maillage.cuf:208 */
    const std::string mpath = trim(C->meshfile_path), mfile = trim(C->meshfile);
    if (mfile.empty()) rc = io_fail(CF_EINVAL, "namelist: no meshfile");
    else if (!C->is_cgns) rc = read_mesh(join_path(d, mpath + mfile), *C);
    else rc = read_cgns(join_path(d, mpath + mfile), *C);
  }
  if (rc == CF_OK) fill_mesh(*C);
  if (rc == CF_OK && C->solinit == 1)
    rc = read_state_file(join_path(d, trim(C->fich_sol_init)), C->mesh.nelt, C->U0, C->tc_init);
  if (rc != CF_OK) return rc;
  *out = C.release();
  return CF_OK;
}

void cf_case_free(cf_case* c) { delete c; }

const char* cf_case_last_error(void) { return g_io_error.c_str(); }

int cf_case_get(const cf_case* c, const cf_mesh** mesh, const cf_params** params, cf_ic* ic, double* ts,
                int32_t* solinit) {
  if (!c) return CF_EINVAL;
  if (mesh) *mesh = &c->mesh;
  if (params) *params = &c->params;
  if (ic) *ic = c->ic;
  if (ts) *ts = c->ts;
  if (solinit) *solinit = c->solinit;
  return CF_OK;
}

int cf_case_initial_state(const cf_case* c, double* hu3, double* t_file) {
  if (!c || !hu3) return CF_EINVAL;
  if (c->solinit != 1) return io_fail(CF_ESTATE, "solinit is not 1: the case starts from its dam line or plane");
  std::memcpy(hu3, c->U0.data(), c->U0.size() * sizeof(double));
  if (t_file) *t_file = c->tc_init;
  return CF_OK;
}

int cf_write_state_file(const char* path, const double* hu3, int32_t nelt, double t) {
  if (!path || !hu3 || nelt < 0) return io_fail(CF_EINVAL, "null argument");
  FILE* f = std::fopen(path, "w");
  if (!f) return io_fail(CF_EINVAL, std::string("cannot write ") + path);
  /* write(*) tc, then '(4f16.6)' per element: three fields of 16 columns, 6 decimals (a value
   * wider than 16 columns prints as asterisks, as Fortran does) */
  std::fprintf(f, " %.17g\n", t);
  char buf[64];
  for (int32_t i = 0; i < nelt; ++i) {
    for (int k = 0; k < 3; ++k) {
      const int n = std::snprintf(buf, sizeof(buf), "%16.6f", hu3[3 * (size_t)i + k]);
      if (n > 16 || !std::isfinite(hu3[3 * (size_t)i + k])) std::fputs("****************", f);
      else std::fputs(buf, f);
    }
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  return ok ? CF_OK : io_fail(CF_EINVAL, std::string("write error on ") + path);
}

}  // extern "C"
