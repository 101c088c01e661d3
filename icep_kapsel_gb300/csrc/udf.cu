// udf.cu -- a minimal reader of the reference's UDF input files (host code).
//
// The reference reads its parameters through OCTA's UDFManager
// (Gourmet_file_io, input.cxx:457-2139), which is not available here. A UDF
// file is a schema ("\begin{global_def}" / "\begin{def}" sections: typed,
// named entries, `class` records, `select` choices, `[]` arrays) and data
// ("\begin{data}": `name: value` entries whose values are positional
// `{...}` records and `[...]` lists, bound to the schema entry by position).
// The input file normally pulls the schema in with \include{"define.udf"}.
// This reader parses both, binds every data value to its dotted path
// ("constitutive_eq.Electrolyte.Dielectric_property.ON.potential_iter",
// "switch.INIT_distribution.user_specify.Particles[3].R.x", as the
// reference's Location paths), and maps the keys of the ICEP path to
// icep_params and the initial particles (udf_to_params below).
#include <ctype.h>
#include <errno.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/icep_gb300.h"

namespace icep {
namespace udf {

// ---- tokens -----------------------------------------------------------------
enum TokKind { T_END = 0, T_PUNCT, T_STRING, T_WORD, T_DIRECTIVE };
struct Tok {
  TokKind k;
  std::string s;  // punctuation char, string contents, word, directive name
  std::string arg;  // directive argument ({...} contents)
  int line;
};

static bool lex(const std::string &src, std::vector<Tok> &out, std::string &err) {
  size_t i = 0, n = src.size();
  int line = 1;
  while (i < n) {
    const char c = src[i];
    if (c == '\n') { line++; i++; continue; }
    if (c == ' ' || c == '\t' || c == '\r' || c == ',' || c == ';') { i++; continue; }
    if (c == '/' && i + 1 < n && src[i + 1] == '/') {
      while (i < n && src[i] != '\n') i++;
      continue;
    }
    if (c == '/' && i + 1 < n && src[i + 1] == '*') {
      i += 2;
      while (i + 1 < n && !(src[i] == '*' && src[i + 1] == '/')) {
        if (src[i] == '\n') line++;
        i++;
      }
      i += 2;
      continue;
    }
    if (c == '{' || c == '}' || c == '[' || c == ']' || c == ':') {
      out.push_back(Tok{T_PUNCT, std::string(1, c), "", line});
      i++;
      continue;
    }
    if (c == '"' || c == '\'') {
      const char q = c;
      size_t j = i + 1;
      std::string v;
      while (j < n && src[j] != q) {
        if (src[j] == '\n') line++;
        v += src[j++];
      }
      if (j >= n) {
        err = "unterminated string at line " + std::to_string(line);
        return false;
      }
      out.push_back(Tok{T_STRING, v, "", line});
      i = j + 1;
      continue;
    }
    if (c == '\\') {  // \begin{...}, \end{...}, \include{...}
      size_t j = i + 1;
      std::string name;
      while (j < n && isalpha((unsigned char)src[j])) name += src[j++];
      std::string arg;
      if (j < n && src[j] == '{') {
        size_t k = j + 1;
        while (k < n && src[k] != '}') arg += src[k++];
        j = (k < n) ? k + 1 : k;
      }
      // strip quotes and blanks of the argument
      std::string a;
      for (char ch : arg)
        if (ch != '"' && ch != '\'' && ch != ' ' && ch != '\t') a += ch;
      out.push_back(Tok{T_DIRECTIVE, name, a, line});
      i = j;
      continue;
    }
    // a bare word: a name, a type or a number
    size_t j = i;
    std::string w;
    while (j < n) {
      const char d = src[j];
      if (d == ' ' || d == '\t' || d == '\r' || d == '\n' || d == ',' || d == ';' || d == '{' || d == '}' ||
          d == '[' || d == ']' || d == ':' || d == '"' || d == '\'')
        break;
      if (d == '/' && j + 1 < n && (src[j + 1] == '/' || src[j + 1] == '*')) break;
      w += d;
      j++;
    }
    if (w.empty()) {
      err = std::string("unexpected character '") + c + "' at line " + std::to_string(line);
      return false;
    }
    out.push_back(Tok{T_WORD, w, "", line});
    i = j;
  }
  return true;
}

// ---- schema -----------------------------------------------------------------
struct Type;
struct Field {
  std::string name;
  int dims = 0;  // number of [] after the name
  std::shared_ptr<Type> type;
};
enum TypeKind { K_SCALAR, K_STRING, K_SELECT, K_STRUCT, K_CLASS };
struct Type {
  TypeKind k = K_SCALAR;
  std::vector<std::string> options;  // select
  std::vector<Field> fields;         // struct
  std::string cls;                   // class reference (resolved at bind time)
};

// ---- data -------------------------------------------------------------------
struct Value {
  bool list = false;
  char open = 0;      // '{' or '[' for lists
  std::string text;   // scalar text
  bool quoted = false;
  std::vector<Value> items;
};

// ---- parser -----------------------------------------------------------------
class Parser {
 public:
  std::map<std::string, Field> globals;                // top-level schema entries
  std::map<std::string, std::shared_ptr<Type>> classes;
  std::vector<std::pair<std::string, Value>> data;     // top-level data entries, in order
  std::string err;

  bool parse_file(const std::string &path, int depth = 0) {
    if (depth > 8) return fail("\\include nesting too deep");
    std::ifstream in(path);
    if (!in) return fail("cannot open " + path);
    std::stringstream ss;
    ss << in.rdbuf();
    std::vector<Tok> toks;
    if (!lex(ss.str(), toks, err)) {
      err = path + ": " + err;
      return false;
    }
    toks.push_back(Tok{T_END, "", "", 0});
    const std::string dir = path.find('/') == std::string::npos ? "" : path.substr(0, path.rfind('/') + 1);
    size_t i = 0;
    // sections: header (skipped), global_def / def (schema), data
    while (toks[i].k != T_END) {
      const Tok &t = toks[i];
      if (t.k == T_DIRECTIVE && t.s == "include") {
        std::string inc = t.arg;
        if (!inc.empty() && inc[0] != '/') inc = dir + inc;
        if (!parse_file(inc, depth + 1)) return false;
        i++;
      } else if (t.k == T_DIRECTIVE && t.s == "begin") {
        const std::string sec = t.arg;
        i++;
        if (sec == "header") {
          while (toks[i].k != T_END && !(toks[i].k == T_DIRECTIVE && toks[i].s == "end" && toks[i].arg == "header")) i++;
          if (toks[i].k != T_END) i++;
        } else if (sec == "global_def" || sec == "def") {
          if (!schema_entries(toks, i, nullptr, sec)) return false;
        } else if (sec == "data") {
          if (!data_entries(toks, i)) return false;
        } else {
          return fail("unknown section " + sec + " in " + path);
        }
      } else {
        return fail(path + ": unexpected token '" + t.s + "' at line " + std::to_string(t.line));
      }
    }
    return true;
  }

 private:
  bool fail(const std::string &m) {
    err = m;
    return false;
  }
  static bool is_p(const Tok &t, char c) { return t.k == T_PUNCT && t.s[0] == c; }

  // entries until '}' (inside a struct) or \end{sec} (top level)
  bool schema_entries(const std::vector<Tok> &toks, size_t &i, std::vector<Field> *into, const std::string &sec) {
    while (true) {
      const Tok &t = toks[i];
      if (t.k == T_END) return into ? fail("unterminated schema record") : fail("unterminated section " + sec);
      if (into && is_p(t, '}')) {
        i++;
        return true;
      }
      if (!into && t.k == T_DIRECTIVE && t.s == "end") {
        i++;
        return true;
      }
      if (t.k == T_STRING) {  // a description after an entry
        i++;
        continue;
      }
      bool is_class = false;
      if (t.k == T_WORD && t.s == "class") {
        is_class = true;
        i++;
      }
      if (toks[i].k != T_WORD) return fail("schema: expected a name at line " + std::to_string(toks[i].line));
      Field f;
      f.name = toks[i].s;
      i++;
      while (is_p(toks[i], '[') && is_p(toks[i + 1], ']')) {
        f.dims++;
        i += 2;
      }
      if (!is_p(toks[i], ':')) return fail("schema: expected ':' after " + f.name);
      i++;
      if (!schema_type(toks, i, f.type)) return false;
      if (is_class) classes[f.name] = f.type;
      else if (into) into->push_back(f);
      else globals[f.name] = f;
    }
  }

  bool schema_type(const std::vector<Tok> &toks, size_t &i, std::shared_ptr<Type> &ty) {
    ty = std::make_shared<Type>();
    const Tok &t = toks[i];
    if (is_p(t, '{')) {
      i++;
      ty->k = K_STRUCT;
      return schema_entries(toks, i, &ty->fields, "");
    }
    if (t.k != T_WORD) return fail("schema: expected a type at line " + std::to_string(t.line));
    i++;
    if (t.s == "select") {
      ty->k = K_SELECT;
      if (!is_p(toks[i], '{')) return fail("schema: select without options");
      i++;
      while (toks[i].k == T_STRING) ty->options.push_back(toks[i++].s);
      if (!is_p(toks[i], '}')) return fail("schema: bad select options at line " + std::to_string(toks[i].line));
      i++;
    } else if (t.s == "int" || t.s == "double" || t.s == "float" || t.s == "bool") {
      ty->k = K_SCALAR;
    } else if (t.s == "string") {
      ty->k = K_STRING;
    } else {
      ty->k = K_CLASS;
      ty->cls = t.s;
    }
    return true;
  }

  bool data_value(const std::vector<Tok> &toks, size_t &i, Value &v) {
    const Tok &t = toks[i];
    if (is_p(t, '{') || is_p(t, '[')) {
      const char close = t.s[0] == '{' ? '}' : ']';
      v.list = true;
      v.open = t.s[0];
      i++;
      while (!is_p(toks[i], close)) {
        if (toks[i].k == T_END) return fail("data: unterminated record");
        Value c;
        if (!data_value(toks, i, c)) return false;
        v.items.push_back(c);
      }
      i++;
      return true;
    }
    if (t.k == T_STRING || t.k == T_WORD) {
      v.text = t.s;
      v.quoted = t.k == T_STRING;
      i++;
      return true;
    }
    return fail("data: unexpected token '" + t.s + "' at line " + std::to_string(t.line));
  }

  bool data_entries(const std::vector<Tok> &toks, size_t &i) {
    while (true) {
      const Tok &t = toks[i];
      if (t.k == T_END) return fail("unterminated data section");
      if (t.k == T_DIRECTIVE && t.s == "end") {
        i++;
        return true;
      }
      if (t.k != T_WORD || !is_p(toks[i + 1], ':'))
        return fail("data: expected 'name:' at line " + std::to_string(t.line));
      const std::string name = t.s;
      i += 2;
      Value v;
      if (!data_value(toks, i, v)) return false;
      data.emplace_back(name, v);
    }
  }
};

// ---- binding: every data value to its dotted path ------------------------------
class Bound {
 public:
  std::map<std::string, std::string> kv;
  std::string err;

  bool bind_all(const Parser &ps) {
    for (const auto &e : ps.data) {
      auto it = ps.globals.find(e.first);
      if (it == ps.globals.end()) {
        err = "data entry '" + e.first + "' has no definition";
        return false;
      }
      if (!bind(ps, *it->second.type, it->second.dims, e.second, e.first)) return false;
    }
    return true;
  }
  bool has(const std::string &k) const { return kv.count(k) != 0; }
  bool str(const std::string &k, std::string &v) {
    auto it = kv.find(k);
    if (it == kv.end()) return fail("missing key " + k);
    v = it->second;
    return true;
  }
  bool num(const std::string &k, double &v) {
    std::string t;
    if (!str(k, t)) return false;
    char *end = nullptr;
    errno = 0;
    v = strtod(t.c_str(), &end);
    if (end == t.c_str() || *end != 0 || errno == ERANGE) return fail("key " + k + ": not a number: " + t);
    return true;
  }
  bool integer(const std::string &k, int &v) {
    double d;
    if (!num(k, d)) return false;
    if (d != std::floor(d) || std::fabs(d) > 2147483647.0) return fail("key " + k + ": not an integer");
    v = (int)d;
    return true;
  }
  bool fail(const std::string &m) {
    err = m;
    return false;
  }

 private:
  bool bind(const Parser &ps, const Type &ty, int dims, const Value &v, const std::string &path) {
    if (dims > 0) {
      if (!v.list || v.open != '[') return fail(path + ": expected a [...] list");
      for (size_t q = 0; q < v.items.size(); q++)
        if (!bind(ps, ty, dims - 1, v.items[q], path + "[" + std::to_string(q) + "]")) return false;
      kv[path + ".size"] = std::to_string(v.items.size());
      return true;
    }
    const Type *t = &ty;
    if (t->k == K_CLASS) {
      auto it = ps.classes.find(t->cls);
      if (it == ps.classes.end()) return fail(path + ": unknown type " + t->cls);
      t = it->second.get();
    }
    if (t->k == K_STRUCT) {
      if (!v.list || v.open != '{') return fail(path + ": expected a {...} record");
      if (v.items.size() > t->fields.size()) return fail(path + ": more values than the record has fields");
      for (size_t q = 0; q < v.items.size(); q++) {
        const Field &f = t->fields[q];
        if (!bind(ps, *f.type, f.dims, v.items[q], path + "." + f.name)) return false;
      }
      return true;
    }
    if (v.list) return fail(path + ": expected a single value");
    if (t->k == K_SELECT) {
      bool ok = false;
      for (const auto &o : t->options) ok = ok || o == v.text;
      if (!ok) return fail(path + ": '" + v.text + "' is not one of its choices");
    }
    kv[path] = v.text;
    return true;
  }
};

// ---- the ICEP path's keys -> icep_params (Gourmet_file_io, input.cxx:457-2139;
// Set_global_parameters, input.cxx:286-440) -------------------------------------
struct Result {
  icep_params p;
  std::vector<icep_particle> parts;
  int gts = 0, num_snap = 0;
  int status = ICEP_OK;
  std::string err;
};

static bool unsupported(Result &r, const std::string &m) {
  r.status = ICEP_ERR_UNSUPPORTED;
  r.err = m;
  return false;
}
static bool bad(Result &r, Bound &b) {
  r.status = ICEP_ERR_ARG;
  r.err = b.err;
  return false;
}

// glibc's rand() sequence (srand(seed)) from a private state, so that the
// caller's rand() state is untouched: the reference seeds rand() with 10
// before placing particles (SRA(GIVEN_SEED, 10), init_particle.cxx:18)
struct Rand {
  struct random_data rd;
  char state[128];
  explicit Rand(unsigned seed) {
    memset(&rd, 0, sizeof(rd));
    memset(state, 0, sizeof(state));
    initstate_r(seed, state, sizeof(state), &rd);
  }
  int next() {
    int32_t v = 0;
    random_r(&rd, &v);
    return (int)v;
  }
  double ax(double x) { return (double)next() / RAND_MAX * x; }                   // RAx, macro.h:83-85
  double ra() { return 2.0 * ((double)next() - RAND_MAX * 0.5) / (RAND_MAX); }   // RA, macro.h:80-82
};

static bool fill(Bound &b, Result &r) {
  icep_params &p = r.p;
  memset(&p, 0, sizeof(p));
  std::string eq;
  if (!b.str("constitutive_eq.type", eq)) return bad(r, b);
  if (eq == "Navier_Stokes") p.sw_eq = ICEP_NAVIER_STOKES;
  else if (eq == "Electrolyte") p.sw_eq = ICEP_ELECTROLYTE;
  else return unsupported(r, "constitutive_eq " + eq + " is not on this path");
  const std::string ce = "constitutive_eq." + eq + ".";
  if (!b.num(ce + "DX", p.dx) || !b.num(ce + "RHO", p.rho) || !b.num(ce + "ETA", p.eta) || !b.num(ce + "kBT", p.kbt))
    return bad(r, b);
  p.dielectric_cst = 1.0;
  p.elementary_charge = 1.0;  // Elementary_charge (input.cxx:254)
  double max_onsager = 0.0;
  if (p.sw_eq == ICEP_ELECTROLYTE) {
    std::string v;
    if (!b.num(ce + "Dielectric_cst", p.dielectric_cst) || !b.str(ce + "INIT_profile", v)) return bad(r, b);
    // INIT_profile (input.cxx:704-715); the engine refuses the relaxations
    // it does not build (salt-free, a single particle in salt)
    if (v == "Uniform") p.poisson_boltzmann = 0;
    else if (v == "Poisson_Boltzmann") p.poisson_boltzmann = 1;
    else return bad(r, b);
    if (!b.str(ce + "Dielectric_property.type", v)) return bad(r, b);
    if (v != "ON") return unsupported(r, "Electrolyte with Dielectric_property OFF");
    p.dielectric = 1;
    const std::string dp = ce + "Dielectric_property.ON.";
    if (!b.integer(dp + "potential_iter", p.potential_iter) || !b.num(dp + "potential_tol", p.potential_tol) ||
        !b.num(dp + "fluid", p.eps_fluid) || !b.num(dp + "particle_top", p.eps_particle_top) ||
        !b.num(dp + "particle_bottom", p.eps_particle_bottom))
      return bad(r, b);
    if (!b.str(ce + "Add_salt.type", v)) return bad(r, b);
    if (v == "saltfree") {  // N_spec = 1: the counterions only (input.cxx:756-766)
      const std::string sf = ce + "Add_salt.saltfree.";
      p.salt_free = 1;
      if (!b.num(sf + "Valency_counterion", p.valency_counterion) ||
          !b.num(sf + "Onsager_coeff_counterion", p.onsager_counterion))
        return bad(r, b);
      max_onsager = p.onsager_counterion;
    } else if (v == "salt") {
      const std::string sa = ce + "Add_salt.salt.";
      if (!b.num(sa + "Valency_positive_ion", p.valency_pos) || !b.num(sa + "Valency_negative_ion", p.valency_neg) ||
          !b.num(sa + "Onsager_coeff_positive_ion", p.onsager_pos) ||
          !b.num(sa + "Onsager_coeff_negative_ion", p.onsager_neg) || !b.num(sa + "Debye_length", p.debye_length))
        return bad(r, b);
      max_onsager = p.onsager_pos > p.onsager_neg ? p.onsager_pos : p.onsager_neg;
    } else {
      return bad(r, b);
    }
    if (!b.str(ce + "Electric_field.type", v)) return bad(r, b);
    if (v == "ON") {
      if (!b.str(ce + "Electric_field.ON.type", v)) return bad(r, b);
      if (v != "DC" && v != "AC") return bad(r, b);
      // DC: E_ext; AC: E_ext sin(2 pi Frequency t) (input.cxx:812-855)
      const std::string ef = ce + "Electric_field.ON." + v + ".";
      p.external_field = 1;
      p.ac = v == "AC" ? 1 : 0;
      if (!b.num(ef + "Ex", p.e_ext[0]) || !b.num(ef + "Ey", p.e_ext[1]) || !b.num(ef + "Ez", p.e_ext[2]))
        return bad(r, b);
      if (p.ac && !b.num(ef + "Frequency", p.frequency)) return bad(r, b);
    }
  }
  // particles (object_type.spherical_particle, input.cxx:878-1100)
  std::string ot;
  if (!b.str("object_type.type", ot)) return bad(r, b);
  if (ot != "spherical_particle") return unsupported(r, "object_type " + ot);
  int nspec = 0;
  {
    std::string n;
    if (b.str("object_type.spherical_particle.Particle_spec.size", n)) nspec = atoi(n.c_str());
  }
  if (nspec < 1 || nspec > ICEP_MAX_SPECIES) return unsupported(r, "number of particle species out of range 1..4");
  p.n_species = nspec;
  std::vector<int> counts((size_t)nspec);
  for (int i = 0; i < nspec; i++) {
    const std::string ps = "object_type.spherical_particle.Particle_spec[" + std::to_string(i) + "].";
    double charge = 0.0;
    std::string ax, prop;
    if (!b.integer(ps + "Particle_number", counts[i]) || !b.num(ps + "MASS_RATIO", p.mass_ratio[i]) ||
        !b.num(ps + "Surface_charge", charge) || !b.str(ps + "janus_axis", ax) || !b.str(ps + "janus_propulsion", prop))
      return bad(r, b);
    if (counts[i] < 0) return unsupported(r, "negative Particle_number");
    p.surface_charge[i] = (p.sw_eq == ICEP_ELECTROLYTE) ? charge : 0.0;
    if (p.sw_eq == ICEP_ELECTROLYTE && (charge != 0.0) != (p.surface_charge[0] != 0.0)) {
      r.status = ICEP_ERR_ARG;  // Init_rho_ion_dielectric (operate_electrolyte.cxx:912-930)
      r.err = "Surface_charge must be non-zero for every species or for none";
      return false;
    }
    p.janus_axis[i] = ax == "X" ? ICEP_JANUS_X : ax == "Y" ? ICEP_JANUS_Y : ax == "Z" ? ICEP_JANUS_Z : ICEP_JANUS_NONE;
    if (prop == "OFF") {
      p.janus_propulsion[i] = ICEP_NO_PROPULSION;
    } else if (prop == "TUMBLER") {
      p.janus_propulsion[i] = ICEP_MOTOR;
      for (int d = 0; d < 3; d++) {
        const char *xyz[3] = {"x", "y", "z"};
        if (!b.num(ps + "janus_force." + xyz[d], p.janus_force[i][d]) ||
            !b.num(ps + "janus_torque." + xyz[d], p.janus_torque[i][d]))
          return bad(r, b);
      }
    } else {
      return unsupported(r, "janus_propulsion " + prop);
    }
    p.n_particles += counts[i];
  }
  if (!b.num("A_XI", p.a_xi) || !b.num("A", p.a) || !b.num("gravity.G", p.g) || !b.num("EPSILON", p.lj_epsilon))
    return bad(r, b);
  {
    std::string gd, lj;
    if (!b.str("gravity.G_direction", gd) || !b.str("LJ_powers", lj)) return bad(r, b);
    p.g_direction = gd == "-X" ? 0 : gd == "-Y" ? 1 : 2;
    p.lj_powers = lj == "12:6" ? 0 : lj == "24:12" ? 1 : 2;
  }
  int np3[3];
  if (!b.integer("mesh.NPX", np3[0]) || !b.integer("mesh.NPY", np3[1]) || !b.integer("mesh.NPZ", np3[2]))
    return bad(r, b);
  for (int d = 0; d < 3; d++)
    if (np3[d] < 4 || np3[d] > 8) return unsupported(r, "mesh exponents must lie in 4..8 (16..256 points)");
  p.nx = 1 << np3[0];
  p.ny = 1 << np3[1];
  p.nz = 1 << np3[2];
  {  // time_increment: manual, or auto = factor * Tdump (input.cxx:333-398)
    std::string ti;
    if (!b.str("time_increment.type", ti)) return bad(r, b);
    if (ti == "manual") {
      if (!b.num("time_increment.manual.delta_t", p.dt)) return bad(r, b);
    } else {
      double factor;
      if (!b.num("time_increment.auto.factor", factor)) return bad(r, b);
      const int N[3] = {p.nx, p.ny, p.nz};
      double kmax2 = 0.0;
      for (int d = 0; d < 3; d++) {
        const double wave = 2.0 * M_PI / (N[d] * p.dx);
        const int trn = (N[d] + 2) / 3;
        kmax2 += (wave * trn) * (wave * trn);
      }
      const double nu = p.eta * (1. / p.rho);
      double tdump = 1. / (nu * kmax2);
      if (p.sw_eq == ICEP_ELECTROLYTE) {
        const double diffusion_time = 1. / (p.kbt * max_onsager * kmax2);
        tdump = tdump < diffusion_time ? tdump : diffusion_time;
        if (p.external_field && p.ac) {  // a hundredth of the AC period (input.cxx:369-375)
          const double frequency_time = 1. / p.frequency;
          const double t_ac = 1.e-2 * frequency_time;
          tdump = tdump < t_ac ? tdump : t_ac;
        }
      }
      p.dt = factor * tdump;
    }
  }
  std::string sw;
  if (!b.str("switch.ROTATION", sw)) return bad(r, b);
  p.rotation = sw == "ON" ? 1 : 0;
  if (!b.str("switch.LJ_truncate", sw)) return bad(r, b);
  p.lj_truncate = sw == "ON" ? 1 : sw == "OFF" ? 0 : -1;
  {  // FIX_CELL (input.cxx:1603-1625)
    const char *xyz[3] = {"x", "y", "z"};
    for (int d = 0; d < 3; d++) {
      std::string v;
      if (b.str(std::string("switch.FIX_CELL.") + xyz[d], v) && v == "ON") p.fix_cell |= 1 << d;
    }
  }
  if (b.str("switch.pin.type", sw) && sw == "YES") return unsupported(r, "pinned particles");
  p.precision = ICEP_FP64;
  p.solver = ICEP_SOLVER_REF;
  if (!b.integer("output.GTS", r.gts) || !b.integer("output.Num_snap", r.num_snap)) return bad(r, b);
  if (b.str("resume.Calculation", sw) && sw == "CONTINUE")
    return unsupported(r, "resume.Calculation CONTINUE (restart from an icep checkpoint file instead)");
  return true;
}

// Initial particles (Init_Particle, init_particle.cxx:12-420): species in
// order, positions uniform_random (rand() seeded with 10, a new draw while
// the periodic distance to an earlier particle is <= 1.05 SIGMA) or
// user_specify (R, v, q, omega); orientations random (RA_on_sphere4D from
// the same sequence), space_align or the user's; velocities zero unless
// user-specified.
static bool init_particles(Bound &b, Result &r) {
  const icep_params &p = r.p;
  const int n = p.n_particles;
  r.parts.assign((size_t)n, icep_particle());
  memset(r.parts.data(), 0, sizeof(icep_particle) * (size_t)n);
  {
    int i = 0;
    for (int sp = 0; sp < p.n_species; sp++) {
      int cnt = 0;
      b.integer("object_type.spherical_particle.Particle_spec[" + std::to_string(sp) + "].Particle_number", cnt);
      for (int k = 0; k < cnt; k++) r.parts[(size_t)i++].spec = sp;
    }
  }
  std::string dist, orient;
  if (!b.str("switch.INIT_distribution.type", dist) || !b.str("switch.INIT_orientation", orient)) return bad(r, b);
  const double L[3] = {p.nx * p.dx, p.ny * p.dx, p.nz * p.dx};
  Rand rng(10);
  if (dist == "uniform_random") {
    const double overlap = 2.0 * p.a * p.dx * 1.05;
    const long max_draws = 10000000L;
    long draws = 0;
    for (int i = 0; i < n; i++) {
      while (true) {
        if (++draws > max_draws) return unsupported(r, "uniform_random placement: no room for the particles");
        double *x = r.parts[(size_t)i].x;
        for (int d = 0; d < 3; d++) x[d] = rng.ax(L[d]);
        int j = 0;
        for (; j < i; j++) {  // Distance0 (interaction.h:122-135)
          double s2 = 0.0;
          for (int d = 0; d < 3; d++) {
            double x12 = r.parts[(size_t)j].x[d] - x[d];
            const double q = x12 / L[d];
            x12 -= (double)(q >= 0.0 ? (int)(q + 0.5) : (int)(q - 0.5)) * L[d];
            s2 += x12 * x12;
          }
          if (sqrt(s2) <= overlap) break;
        }
        if (j >= i) break;
      }
    }
  } else if (dist == "user_specify") {
    std::string cnt;
    if (!b.str("switch.INIT_distribution.user_specify.Particles.size", cnt) || atoi(cnt.c_str()) < n)
      return unsupported(r, "user_specify lists fewer particles than Particle_number");
    const char *xyz[3] = {"x", "y", "z"};
    for (int i = 0; i < n; i++) {
      const std::string t = "switch.INIT_distribution.user_specify.Particles[" + std::to_string(i) + "].";
      icep_particle &q = r.parts[(size_t)i];
      for (int d = 0; d < 3; d++)
        if (!b.num(t + "R." + xyz[d], q.x[d]) || !b.num(t + "v." + xyz[d], q.v[d]) ||
            !b.num(t + "omega." + xyz[d], q.omega[d]))
          return bad(r, b);
      for (int a = 0; a < 4; a++)
        if (!b.num(t + "q.q" + std::to_string(a), q.q[a])) return bad(r, b);
      if (!(p.rotation && orient == "user_specify")) {
        q.q[0] = 1.0;
        q.q[1] = q.q[2] = q.q[3] = 0.0;
      } else {
        // qtn_normalize (quaternion.h:283-291)
        const double nq = sqrt(q.q[0] * q.q[0] + q.q[1] * q.q[1] + q.q[2] * q.q[2] + q.q[3] * q.q[3]);
        if (!(nq > 0.0)) return unsupported(r, "user_specify: zero quaternion");
        const double inv = 1.0 / nq;
        for (int a = 0; a < 4; a++) q.q[a] *= inv;
      }
    }
  } else {
    return unsupported(r, "INIT_distribution " + dist);
  }
  for (int i = 0; i < n; i++) {
    icep_particle &q = r.parts[(size_t)i];
    for (int d = 0; d < 3; d++) q.x_nopbc[d] = q.x[d];
    if (dist != "user_specify") q.q[0] = 1.0;
    if (p.rotation && orient == "random") {  // random_rqtn (quaternion.h:468-473)
      double u0, u1, u2, u3;
      do {
        u0 = rng.ra();
        u1 = rng.ra();
      } while (!(u0 * u0 + u1 * u1 <= 1));
      do {
        u2 = rng.ra();
        u3 = rng.ra();
      } while (!(u2 * u2 + u3 * u3 <= 1));
      const double scale = sqrt((1.0 - (u0 * u0 + u1 * u1)) / (u2 * u2 + u3 * u3));
      q.q[0] = u0;
      q.q[1] = u1;
      q.q[2] = u2 * scale;
      q.q[3] = u3 * scale;
    }
    for (int a = 0; a < 4; a++) q.q_old[a] = q.q[a];
  }
  return true;
}

static bool read_udf(const char *path, Result &r, Bound *keep = nullptr) {
  Parser ps;
  if (!ps.parse_file(path)) {
    r.status = ICEP_ERR_ARG;
    r.err = ps.err;
    return false;
  }
  Bound b;
  if (!b.bind_all(ps)) return bad(r, b);
  if (keep) {
    *keep = b;
    return true;
  }
  return fill(b, r) && init_particles(b, r);
}

static void copy_err(const std::string &m, char *err, int len) {
  if (!err || len <= 0) return;
  const size_t n = m.size() < (size_t)(len - 1) ? m.size() : (size_t)(len - 1);
  memcpy(err, m.data(), n);
  err[n] = 0;
}

}  // namespace udf
}  // namespace icep

extern "C" {

int icep_udf_read(const char *path, icep_params *params, icep_particle *particles, int max_particles,
                  int *n_particles, int *gts, int *num_snap, char *err, int err_len) {
  icep::udf::copy_err("", err, err_len);
  if (!path || !params) return ICEP_ERR_ARG;
  icep::udf::Result r;
  if (!icep::udf::read_udf(path, r)) {
    icep::udf::copy_err(r.err, err, err_len);
    return r.status;
  }
  *params = r.p;
  if (n_particles) *n_particles = r.p.n_particles;
  if (gts) *gts = r.gts;
  if (num_snap) *num_snap = r.num_snap;
  if (particles) {
    if (max_particles < r.p.n_particles) {
      icep::udf::copy_err("particle array too small", err, err_len);
      return ICEP_ERR_ARG;
    }
    memcpy(particles, r.parts.data(), sizeof(icep_particle) * (size_t)r.p.n_particles);
  }
  return ICEP_OK;
}

int icep_udf_value(const char *path, const char *key, char *value, int len) {
  if (!path || !key || !value || len <= 0) return ICEP_ERR_ARG;
  icep::udf::Result r;
  icep::udf::Bound b;
  if (!icep::udf::read_udf(path, r, &b)) {
    icep::udf::copy_err(r.err, value, len);
    return r.status;
  }
  std::string v;
  if (!b.str(key, v)) {
    icep::udf::copy_err(b.err, value, len);
    return ICEP_ERR_ARG;
  }
  if ((int)v.size() >= len) return ICEP_ERR_ARG;
  icep::udf::copy_err(v, value, len);
  return ICEP_OK;
}

}  // extern "C"
