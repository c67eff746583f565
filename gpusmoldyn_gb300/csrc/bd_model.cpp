// bd_model.cpp -- a handle from a model written in a subset of Smoldyn's
// configuration language, in place of the reference's hard-coded presets
// (ParticleSystem::test1Reactions .. test3Types, particleSystem.cpp:319-571,
// whose comments quote the same statements, e.g. "reaction fwd E + S -> ES
// 0.01" and "product_placement back pgemmax 0.2" at :400-403).
//
// Accepted statements (one per line, '#' starts a comment):
//   dim 3
//   boundaries <axis> <low> <high> [r]       axis 0|1|2|x|y|z, reflecting walls
//   low_wall <axis> <pos> r / high_wall <axis> <pos> r
//   species <name> ...
//   difc <species>[(state)]|all <D>
//   time_start <t> / time_stop <t> / time_step <dt>
//   random_seed <n>
//   reaction <name> <r1> [+ <r2>] -> <p1> [+ <p2>] <rate>     "0" = none
//   reaction_rate <name> <rate>
//   reaction_probability <name> <p>
//   product_placement <name> irrev|pgem|pgemmax|unbindrad [<value>]
//   mol <count> <species> <x|u> <y|u> <z|u>  u = uniform in the box
//   start_surface <name> ... end_surface, with inside:
//     action <species|all> <front|back|both> <reflect|absorb|transmit>
//       (the face may also come first)
//     panel rect <+-axis> <x> <y> <z> <side1> <side2>
//     panel tri <x1> <y1> <z1> <x2> <y2> <z2> <x3> <y3> <z3>
//     panel sph <x> <y> <z> <radius>                     (radius < 0: front inside)
//     panel cyl <x1> <y1> <z1> <x2> <y2> <z2> <radius>   (radius < 0: front inside)
//     panel hemi <x> <y> <z> <radius> <ox> <oy> <oz>     (radius < 0: front inside)
//     panel disk <x> <y> <z> <radius> <nx> <ny> <nz>
//     (drawing parameters and panel names after these are ignored)
//   surface <name> <statement>                 one surface statement outside a block
//   end_file
// Display, output and runtime-command statements (graphics, output_files,
// cmd, ...) are accepted and ignored; anything else is an error naming the
// line.  Molecules placed with "u" come from a splitmix64 stream seeded with
// random_seed, so a model text always gives the same initial state.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gpusmoldyn.h"
#include "bd_surface.h"

namespace {

struct RxnStmt {
  std::string name;
  std::vector<std::string> reactants, products;
  double rate = 0.0;
  bool has_rate = false;
  int line = 0;
};

struct MolStmt {
  uint64_t count = 0;
  std::string species;
  std::string coord[3];
  int line = 0;
};

struct ActionStmt {
  std::string species;  // "all" = every species
  int face = BD_FACE_BOTH, action = BD_SURF_REFLECT, line = 0;
};

struct SurfaceStmt {
  std::string name;
  std::vector<ActionStmt> actions;
  std::vector<std::pair<bd_panel, int>> panels;  // panel, line
};

struct Model {
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  bool axis_set[3] = {false, false, false};
  double dt = 0.0, t_start = 0.0, t_stop = 0.0;
  uint64_t seed = 1;
  std::vector<std::string> species;
  std::vector<std::pair<std::string, double>> difc;  // in order; "all" = every species
  std::vector<RxnStmt> rxns;
  std::map<std::string, double> probability;
  std::map<std::string, std::pair<std::string, double>> placement;
  std::vector<MolStmt> mols;
  std::vector<SurfaceStmt> surfaces;
};

const char* const kIgnored[] = {
    "graphics", "graphic_iter", "graphic_delay", "frame_thickness", "frame_color", "grid_thickness",
    "grid_color", "background_color", "display_size", "color", "text_display", "text_color", "light",
    "quit_at_end", "output_files", "output_root", "output_precision", "append_files", "output_file_number",
    "output_format", "cmd", "max_mol", "max_species", "molperbox", "boxsize", "accuracy", "gauss_table_size",
    "epsilon", "margin", "neighbor_dist", "tiff_iter", "tiff_name", "tiff_min", "tiff_max", "tiff_first",
    "max_names", "max_rxn"};

bool ignored(const std::string& w) {
  for (const char* k : kIgnored)
    if (w == k) return true;
  return false;
}

bool parse_axis(const std::string& s, int* a) {
  if (s == "0" || s == "x") *a = 0;
  else if (s == "1" || s == "y") *a = 1;
  else if (s == "2" || s == "z") *a = 2;
  else return false;
  return true;
}

bool parse_num(const std::string& s, double* v) {
  char* end = nullptr;
  *v = strtod(s.c_str(), &end);
  return end && *end == '\0' && !s.empty();
}

// species name without a Smoldyn state suffix: "A(all)" -> "A"
std::string base_name(const std::string& s) {
  const size_t p = s.find('(');
  return p == std::string::npos ? s : s.substr(0, p);
}

struct Failure {
  bd_status code;
  std::string msg;
};

#define FAIL(code, line, text)                                           \
  do {                                                                   \
    std::ostringstream _m;                                               \
    if ((line) > 0) _m << "line " << (line) << ": ";                    \
    _m << text;                                                          \
    throw Failure{(code), _m.str()};                                     \
  } while (0)

// Display statements of a surface block.
bool surface_display(const std::string& k) {
  return k == "color" || k == "colour" || k == "thickness" || k == "stipple" || k == "polygon" ||
         k == "shininess" || k == "max_panels";
}

SurfaceStmt& surface_named(Model& m, const std::string& name) {
  for (SurfaceStmt& f : m.surfaces)
    if (f.name == name) return f;
  m.surfaces.push_back(SurfaceStmt{});
  m.surfaces.back().name = name;
  return m.surfaces.back();
}

// One statement of a surface block, w[0] its keyword.
void surface_statement(SurfaceStmt& f, const std::vector<std::string>& w, int ln) {
  const std::string& k = w[0];
  if (surface_display(k)) return;
  if (k == "action") {
    if (w.size() != 4) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "action <species|all> <front|back|both> <action>");
    auto face_of = [](const std::string& t, int* face) {
      if (t == "front") *face = BD_FACE_FRONT;
      else if (t == "back") *face = BD_FACE_BACK;
      else if (t == "both") *face = BD_FACE_BOTH;
      else return false;
      return true;
    };
    ActionStmt a;
    a.line = ln;
    if (face_of(w[1], &a.face)) {
      a.species = base_name(w[2]);
    } else if (face_of(w[2], &a.face)) {
      a.species = base_name(w[1]);
    } else {
      FAIL(BD_ERR_INVALID_ARGUMENT, ln, "action needs a face: front, back or both");
    }
    const std::string& t = w[3];
    if (t == "reflect" || t == "r") a.action = BD_SURF_REFLECT;
    else if (t == "absorb" || t == "a") a.action = BD_SURF_ABSORB;
    else if (t == "transmit" || t == "t") a.action = BD_SURF_TRANSMIT;
    else FAIL(BD_ERR_UNSUPPORTED, ln, "surface action " << t << " is not supported (reflect, absorb, transmit)");
    f.actions.push_back(a);
    return;
  }
  if (k == "panel") {
    if (w.size() < 2) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "panel <shape> <parameters>");
    bd_panel pn{};
    pn.front = 1;
    const std::string& shape = w[1];
    size_t need = 0, first = 2;
    if (shape == "rect") {
      // "+0", "-x", "+y", ...: the perpendicular axis and the way the front looks
      if (w.size() < 3 || w[2].size() != 2 || (w[2][0] != '+' && w[2][0] != '-') ||
          !parse_axis(w[2].substr(1), &pn.axis))
        FAIL(BD_ERR_INVALID_ARGUMENT, ln, "panel rect <+-axis> <x> <y> <z> <side1> <side2>");
      pn.front = w[2][0] == '+' ? 1 : -1;
      pn.shape = BD_PANEL_RECT;
      need = 5;
      first = 3;
    } else if (shape == "tri") {
      pn.shape = BD_PANEL_TRI;
      need = 9;
    } else if (shape == "sph") {
      pn.shape = BD_PANEL_SPH;
      need = 4;
    } else if (shape == "cyl") {
      pn.shape = BD_PANEL_CYL;
      need = 7;
    } else if (shape == "hemi") {
      pn.shape = BD_PANEL_HEMI;
      need = 7;
    } else if (shape == "disk") {
      pn.shape = BD_PANEL_DISK;
      need = 7;
    } else {
      FAIL(BD_ERR_UNSUPPORTED, ln, "panel shape " << shape << " is not supported");
    }
    if (w.size() < first + need) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "panel " << shape << " needs " << need << " numbers");
    for (size_t i = 0; i < need; i++) {
      double v;
      if (!parse_num(w[first + i], &v)) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "bad number " << w[first + i]);
      pn.p[i] = (float)v;
    }
    // a negative radius turns the front face inward
    const int ri = shape == "cyl" ? 6 : 3;
    if ((shape == "sph" || shape == "cyl" || shape == "hemi") && pn.p[ri] < 0) {
      pn.p[ri] = -pn.p[ri];
      pn.front = -1;
    }
    f.panels.push_back({pn, ln});
    return;
  }
  FAIL(BD_ERR_UNSUPPORTED, ln, "surface statement " << k << " is not supported");
}

Model parse(const std::string& text) {
  Model m;
  std::istringstream in(text);
  std::string raw;
  int ln = 0;
  SurfaceStmt* block = nullptr;  // inside start_surface .. end_surface
  while (std::getline(in, raw)) {
    ++ln;
    const size_t hash = raw.find('#');
    if (hash != std::string::npos) raw.resize(hash);
    std::istringstream ws(raw);
    std::vector<std::string> w;
    for (std::string t; ws >> t;) w.push_back(t);
    if (w.empty()) continue;
    const std::string& k = w[0];
    double v;
    if (k == "end_file") break;
    if (block) {
      if (k == "end_surface") block = nullptr;
      else surface_statement(*block, w, ln);
      continue;
    }
    if (ignored(k) || k == "max_surface") continue;
    if (k == "start_surface") {
      if (w.size() != 2) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "start_surface <name>");
      block = &surface_named(m, w[1]);
    } else if (k == "surface") {
      if (w.size() < 3) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "surface <name> <statement>");
      surface_statement(surface_named(m, w[1]), std::vector<std::string>(w.begin() + 2, w.end()), ln);
    } else if (k == "dim") {
      if (w.size() != 2 || w[1] != "3") FAIL(BD_ERR_UNSUPPORTED, ln, "only dim 3 is supported");
    } else if (k == "boundaries") {
      int a;
      double lo, hi;
      if (w.size() < 4 || !parse_axis(w[1], &a) || !parse_num(w[2], &lo) || !parse_num(w[3], &hi) || !(hi > lo))
        FAIL(BD_ERR_INVALID_ARGUMENT, ln, "boundaries <axis> <low> <high> [r]");
      if (w.size() > 4 && w[4] != "r") FAIL(BD_ERR_UNSUPPORTED, ln, "only reflecting walls (r) are supported");
      m.lo[a] = lo;
      m.hi[a] = hi;
      m.axis_set[a] = true;
    } else if (k == "low_wall" || k == "high_wall") {
      int a;
      if (w.size() < 3 || !parse_axis(w[1], &a) || !parse_num(w[2], &v))
        FAIL(BD_ERR_INVALID_ARGUMENT, ln, k << " <axis> <pos> r");
      if (w.size() > 3 && w[3] != "r") FAIL(BD_ERR_UNSUPPORTED, ln, "only reflecting walls (r) are supported");
      (k == "low_wall" ? m.lo : m.hi)[a] = v;
      m.axis_set[a] = true;
    } else if (k == "species") {
      if (w.size() < 2) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "species <name> ...");
      for (size_t i = 1; i < w.size(); i++) {
        for (const std::string& s : m.species)
          if (s == w[i]) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "species " << w[i] << " declared twice");
        m.species.push_back(w[i]);
      }
    } else if (k == "difc") {
      if (w.size() != 3 || !parse_num(w[2], &v) || v < 0) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "difc <species> <D>");
      m.difc.push_back({base_name(w[1]), v});
    } else if (k == "time_start" || k == "time_stop" || k == "time_step") {
      if (w.size() != 2 || !parse_num(w[1], &v)) FAIL(BD_ERR_INVALID_ARGUMENT, ln, k << " <value>");
      (k == "time_start" ? m.t_start : (k == "time_stop" ? m.t_stop : m.dt)) = v;
    } else if (k == "random_seed" || k == "rand_seed") {
      if (w.size() != 2 || !parse_num(w[1], &v) || v < 0) FAIL(BD_ERR_INVALID_ARGUMENT, ln, k << " <n>");
      m.seed = (uint64_t)v;
    } else if (k == "reaction") {
      // reaction <name> <r1> [+ <r2>] -> <p1> [+ <p2>] <rate>
      RxnStmt r;
      r.line = ln;
      size_t i = 1;
      if (w.size() < 5) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "reaction <name> <reactants> -> <products> [rate]");
      r.name = w[i++];
      std::vector<std::string>* side = &r.reactants;
      bool arrow = false;
      for (; i < w.size(); i++) {
        if (w[i] == "->") {
          if (arrow) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "two arrows");
          arrow = true;
          side = &r.products;
          continue;
        }
        if (w[i] == "+") continue;
        if (arrow && i + 1 == w.size() && parse_num(w[i], &v) && w[i] != "0") {
          r.rate = v;
          r.has_rate = true;
          continue;
        }
        if (w[i] == "0") continue;  // no reactant / no product
        side->push_back(base_name(w[i]));
      }
      if (!arrow) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "reaction without ->");
      if (r.reactants.size() > 2 || r.products.size() > 2)
        FAIL(BD_ERR_UNSUPPORTED, ln, "at most two reactants and two products");
      for (const RxnStmt& o : m.rxns)
        if (o.name == r.name) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "reaction " << r.name << " defined twice");
      m.rxns.push_back(r);
    } else if (k == "reaction_rate") {
      if (w.size() != 3 || !parse_num(w[2], &v)) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "reaction_rate <name> <rate>");
      bool found = false;
      for (RxnStmt& r : m.rxns)
        if (r.name == w[1]) {
          r.rate = v;
          r.has_rate = true;
          found = true;
        }
      if (!found) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "unknown reaction " << w[1]);
    } else if (k == "reaction_probability") {
      if (w.size() != 3 || !parse_num(w[2], &v)) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "reaction_probability <name> <p>");
      m.probability[w[1]] = v;
    } else if (k == "product_placement") {
      if (w.size() < 3) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "product_placement <name> <type> [value]");
      double param = 0.0;
      if (w.size() > 3 && !parse_num(w[3], &param)) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "bad value " << w[3]);
      m.placement[w[1]] = {w[2], param};
    } else if (k == "mol") {
      MolStmt mo;
      mo.line = ln;
      if (w.size() != 6 || !parse_num(w[1], &v) || v < 0)
        FAIL(BD_ERR_INVALID_ARGUMENT, ln, "mol <count> <species> <x|u> <y|u> <z|u>");
      mo.count = (uint64_t)v;
      mo.species = base_name(w[2]);
      for (int a = 0; a < 3; a++) mo.coord[a] = w[3 + a];
      m.mols.push_back(mo);
    } else {
      FAIL(BD_ERR_INVALID_ARGUMENT, ln, "unknown statement '" << k << "'");
    }
  }
  if (block) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "start_surface " << block->name << " without end_surface");
  for (int a = 0; a < 3; a++)
    if (!m.axis_set[a] || !(m.hi[a] > m.lo[a])) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "boundaries missing for axis " << a);
  if (!(m.dt > 0)) FAIL(BD_ERR_INVALID_ARGUMENT, ln, "time_step missing");
  return m;
}

uint64_t splitmix64(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int species_id(const Model& m, const std::string& name, int line) {
  for (size_t i = 0; i < m.species.size(); i++)
    if (m.species[i] == name) return (int)i;
  FAIL(BD_ERR_INVALID_ARGUMENT, line, "unknown species " << name);
  return -1;
}

void check(bd_status st, int line, const char* what) {
  if (st != BD_OK) FAIL(st, line, what << ": " << bd_status_string(st));
}

bd_handle build(const Model& m, int device, bd_model_info* info) {
  bd_config cfg;
  bd_config_default(&cfg);
  for (int a = 0; a < 3; a++) {
    cfg.box_lo[a] = (float)m.lo[a];
    cfg.box_hi[a] = (float)m.hi[a];
  }
  cfg.dt = (float)m.dt;
  cfg.seed = m.seed;
  cfg.device = device;
  bd_handle h = nullptr;
  check(bd_create(&cfg, &h), 0, "bd_create");
  try {
    std::vector<double> D(m.species.size(), 0.0);
    for (const auto& d : m.difc) {
      if (d.first == "all") D.assign(D.size(), d.second);
      else D[species_id(m, d.first, 0)] = d.second;
    }
    for (size_t i = 0; i < m.species.size(); i++) {
      int id;
      check(bd_add_species(h, (float)D[i], &id), 0, "species");
      check(bd_set_species_name(h, id, m.species[i].c_str()), 0, "species name");
    }
    for (const RxnStmt& r : m.rxns) {
      if (!r.has_rate) FAIL(BD_ERR_INVALID_ARGUMENT, r.line, "reaction " << r.name << " has no rate");
      int rc[2] = {-1, -1}, pr[2] = {-1, -1};
      for (size_t i = 0; i < r.reactants.size(); i++) rc[i] = species_id(m, r.reactants[i], r.line);
      for (size_t i = 0; i < r.products.size(); i++) pr[i] = species_id(m, r.products[i], r.line);
      int id;
      check(bd_add_reaction(h, (int)r.reactants.size(), rc, pr, (float)r.rate, &id), r.line, "reaction");
      check(bd_set_reaction_name(h, id, r.name.c_str()), r.line, "reaction name");
    }
    int rx_id;
    for (const auto& pl : m.placement) {
      if (bd_find_reaction(h, pl.first.c_str(), &rx_id) != BD_OK)
        FAIL(BD_ERR_INVALID_ARGUMENT, 0, "product_placement of unknown reaction " << pl.first);
      const std::string& t = pl.second.first;
      int kind;
      if (t == "irrev") kind = BD_PP_OFFSET0;
      else if (t == "pgem") kind = BD_PP_PGEM;
      else if (t == "pgemmax") kind = BD_PP_PGEMMAX;
      else if (t == "unbindrad") kind = BD_PP_UNBINDRAD;
      else FAIL(BD_ERR_UNSUPPORTED, 0, "product placement " << t << " is not supported");
      check(bd_set_product_placement(h, rx_id, kind, (float)pl.second.second), 0, "product_placement");
    }
    for (const auto& pr : m.probability) {
      if (bd_find_reaction(h, pr.first.c_str(), &rx_id) != BD_OK)
        FAIL(BD_ERR_INVALID_ARGUMENT, 0, "reaction_probability of unknown reaction " << pr.first);
      check(bd_set_reaction_probability(h, rx_id, (float)pr.second), 0, "reaction_probability");
    }
    for (const SurfaceStmt& f : m.surfaces) {
      int sid;
      check(bd_add_surface(h, &sid), 0, "surface");
      for (const ActionStmt& a : f.actions) {
        const int sp = a.species == "all" ? BD_ALL_SPECIES : species_id(m, a.species, a.line);
        check(bd_set_surface_action(h, sid, sp, a.face, a.action), a.line, "action");
      }
      for (const auto& pl : f.panels) {
        bd_panel_info probe;
        std::string why;
        if (bd::derive_panel(pl.first, sid, &probe, &why)) FAIL(BD_ERR_INVALID_ARGUMENT, pl.second, "panel: " << why);
        check(bd_add_panel(h, sid, &pl.first, nullptr), pl.second, "panel");
      }
    }
    check(bd_finalize(h), 0, "finalize");
    uint64_t n = 0;
    for (const MolStmt& mo : m.mols) n += mo.count;
    std::vector<float> xyz4((size_t)n * 4 + 4, 0.0f);
    std::vector<int> sp((size_t)n + 1, 0);
    uint64_t rng = m.seed, i = 0;
    for (const MolStmt& mo : m.mols) {
      const int s = species_id(m, mo.species, mo.line);
      double fixed[3];
      bool uni[3];
      for (int a = 0; a < 3; a++) {
        uni[a] = mo.coord[a] == "u";
        if (!uni[a] && !parse_num(mo.coord[a], &fixed[a]))
          FAIL(BD_ERR_INVALID_ARGUMENT, mo.line, "bad coordinate " << mo.coord[a]);
        if (!uni[a] && (fixed[a] < m.lo[a] || fixed[a] > m.hi[a]))
          FAIL(BD_ERR_INVALID_ARGUMENT, mo.line, "coordinate " << mo.coord[a] << " outside the box");
      }
      for (uint64_t c = 0; c < mo.count; c++, i++) {
        for (int a = 0; a < 3; a++) {
          float x;
          if (uni[a]) {
            const double u = (double)(splitmix64(&rng) >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
            x = (float)(m.lo[a] + u * (m.hi[a] - m.lo[a]));
            if (x > (float)m.hi[a]) x = (float)m.hi[a];
            if (x < (float)m.lo[a]) x = (float)m.lo[a];
          } else {
            x = (float)fixed[a];
          }
          xyz4[4 * i + a] = x;
        }
        sp[i] = s;
      }
    }
    check(bd_set_particles(h, xyz4.data(), sp.data(), (size_t)n), 0, "molecules");
    if (info) {
      info->time_start = m.t_start;
      info->time_stop = m.t_stop;
      info->n_molecules = n;
      info->n_species = (int)m.species.size();
      info->n_reactions = (int)m.rxns.size();
      info->steps = m.t_stop > m.t_start ? (uint64_t)llround((m.t_stop - m.t_start) / m.dt) : 0;
    }
  } catch (...) {
    bd_destroy(h);
    throw;
  }
  return h;
}

void put_error(char* err, size_t cap, const std::string& msg) {
  if (!err || cap == 0) return;
  snprintf(err, cap, "%s", msg.c_str());
}

}  // namespace

BD_API bd_status bd_create_from_model(const char* text, int device, bd_handle* out, bd_model_info* info, char* err,
                                      size_t err_cap) {
  if (!text || !out) return BD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  put_error(err, err_cap, "");
  try {
    *out = build(parse(text), device, info);
    return BD_OK;
  } catch (const Failure& f) {
    put_error(err, err_cap, f.msg);
    return f.code;
  }
}

BD_API bd_status bd_create_from_model_file(const char* path, int device, bd_handle* out, bd_model_info* info,
                                           char* err, size_t err_cap) {
  if (!path || !out) return BD_ERR_INVALID_ARGUMENT;
  std::ifstream f(path);
  if (!f) {
    put_error(err, err_cap, std::string("cannot read ") + path);
    return BD_ERR_INVALID_ARGUMENT;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  return bd_create_from_model(ss.str().c_str(), device, out, info, err, err_cap);
}
