// ref_shim.cc -- C entry points over the reference's own host-compiled code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build.py (build_ref) together
// with the reference's sources where they lie (src/emt6ro/cell/cell.cu as C++,
// parameters/parameters.cc, state/state.cc, common/random-engine.cc) into
// oracle/_ref/libemt6_ref.so.  Nothing here is shipped; it exists to pin the
// oracle (oracle/emt6_oracle.c) against the reference and to produce the
// reference-CPU-path distribution fixtures.
//
// ReplayRand serves injected draws to the reference's templated functions
// (Site::step<R>, chooseNeighbour<R>, divideCell<R>; site/site.h:62-82,
// simulation/cell-division.h:10-54): uniform() returns the next value,
// normal(p) returns p.stddev * z + p.mean for the next z.
#include <cstdint>
#include <cstring>
#include <random>
#include <string>

#include "emt6ro/cell/cell.h"
#include "emt6ro/common/random-engine.h"
#include "emt6ro/parameters/parameters.h"
#include "emt6ro/simulation/cell-division.h"
#include "emt6ro/site/site.h"
#include "emt6ro/state/state.h"

extern "C" {
#include "emt6_oracle.h"
}

using emt6ro::Cell;
using emt6ro::Parameters;
using emt6ro::Site;

namespace {

struct ReplayRand {
  const float *v;
  int n;
  int i;
  float uniform() { return i < n ? v[i++] : 0.5f; }
  float normal(const Parameters::NormalDistribution &p) {
    float z = i < n ? v[i++] : 0.f;
    return p.stddev * z + p.mean;
  }
};

Parameters toRef(const orc_params *p) {
  Parameters r{};
  r.lattice_dims = emt6ro::Dims(static_cast<int16_t>(p->lattice_height),
                                static_cast<int16_t>(p->lattice_width));
  r.time_step = p->time_step;
  r.diffusion_params.coeffs = {p->diffusion_coeffs[0], p->diffusion_coeffs[1],
                               p->diffusion_coeffs[2]};
  r.diffusion_params.time_step = p->diffusion_time_step;
  for (int m = 0; m < 4; ++m)
    r.metabolism.values[m] = {p->metabolism[m][0], p->metabolism[m][1], p->metabolism[m][2]};
  r.external_levels = {p->external_levels[0], p->external_levels[1], p->external_levels[2]};
  r.death_gi = p->death_gi;
  r.quiescence_gi = p->quiescence_gi;
  r.death_gi_production = p->death_gi_production;
  for (int k = 0; k < 5; ++k)
    r.cycle_times.params[k] = {p->cycle_times[k][0], p->cycle_times[k][1]};
  r.cell_repair.delay_time = {p->delay_time_coeff, p->delay_time_exp_coeff};
  r.cell_repair.survival_prob = {p->survival_prob_coeff, p->survival_prob_exp_coeff};
  r.cell_repair.repair_half_time = p->repair_half_time;
  return r;
}

void fromRef(const Parameters &r, orc_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->lattice_height = r.lattice_dims.height;
  p->lattice_width = r.lattice_dims.width;
  p->time_step = r.time_step;
  p->diffusion_coeffs[0] = r.diffusion_params.coeffs.cho;
  p->diffusion_coeffs[1] = r.diffusion_params.coeffs.ox;
  p->diffusion_coeffs[2] = r.diffusion_params.coeffs.gi;
  p->diffusion_time_step = r.diffusion_params.time_step;
  for (int m = 0; m < 4; ++m) {
    p->metabolism[m][0] = r.metabolism.values[m].cho;
    p->metabolism[m][1] = r.metabolism.values[m].ox;
    p->metabolism[m][2] = r.metabolism.values[m].gi;
  }
  p->external_levels[0] = r.external_levels.cho;
  p->external_levels[1] = r.external_levels.ox;
  p->external_levels[2] = r.external_levels.gi;
  p->death_gi = r.death_gi;
  p->quiescence_gi = r.quiescence_gi;
  p->death_gi_production = r.death_gi_production;
  for (int k = 0; k < 5; ++k) {
    p->cycle_times[k][0] = r.cycle_times.params[k].mean;
    p->cycle_times[k][1] = r.cycle_times.params[k].stddev;
  }
  p->delay_time_coeff = r.cell_repair.delay_time.coeff;
  p->delay_time_exp_coeff = r.cell_repair.delay_time.exp_coeff;
  p->survival_prob_coeff = r.cell_repair.survival_prob.coeff;
  p->survival_prob_exp_coeff = r.cell_repair.survival_prob.exp_coeff;
  p->repair_half_time = r.cell_repair.repair_half_time;
}

Cell toCell(const orc_site *s) {
  Cell c{};
  c.time_in_repair = s->time_in_repair;
  c.irradiation = s->irradiation;
  c.repair_delay_time = s->repair_delay_time;
  c.proliferation_time = s->proliferation_time;
  for (int i = 0; i < 5; ++i) c.cycle_times.times[i] = s->cycle_times[i];
  c.mode = static_cast<Cell::MetabolicMode>(s->mode);
  c.phase = static_cast<Cell::CyclePhase>(s->phase);
  return c;
}

void fromCell(const Cell &c, orc_site *s) {
  s->time_in_repair = c.time_in_repair;
  s->irradiation = c.irradiation;
  s->repair_delay_time = c.repair_delay_time;
  s->proliferation_time = c.proliferation_time;
  for (int i = 0; i < 5; ++i) s->cycle_times[i] = c.cycle_times.times[i];
  s->mode = static_cast<uint8_t>(c.mode);
  s->phase = static_cast<uint8_t>(c.phase);
}

Site toSite(const orc_site *s) {
  Site site{};
  site.substrates = {s->cho, s->ox, s->gi};
  site.cell = toCell(s);
  site.state = static_cast<Site::State>(s->state);
  return site;
}

void fromSite(const Site &site, orc_site *s) {
  s->cho = site.substrates.cho;
  s->ox = site.substrates.ox;
  s->gi = site.substrates.gi;
  fromCell(site.cell, s);
  s->state = static_cast<uint8_t>(site.state);
}

}  // namespace

extern "C" {

// ---- injected-draw entry points (golden vectors) -------------------------
int ref_site_step_replay(orc_site *s, const orc_params *p, uint32_t vac, float dose,
                         const float *draws, int ndraws, int *used) {
  Parameters params = toRef(p);
  Site site = toSite(s);
  ReplayRand rr{draws, ndraws, 0};
  bool ready = site.step(params, static_cast<uint8_t>(vac), dose, rr);
  fromSite(site, s);
  *used = rr.i;
  return ready ? 1 : 0;
}

int ref_update_state(orc_site *s, const orc_params *p, uint32_t vac) {
  Parameters params = toRef(p);
  Cell c = toCell(s);
  emt6ro::Substrates lv{s->cho, s->ox, s->gi};
  bool alive = c.updateState(lv, params, static_cast<uint8_t>(vac));
  fromCell(c, s);
  return alive ? 1 : 0;
}

int ref_progress_clock(orc_site *s, float time_step) {
  Cell c = toCell(s);
  bool changed = c.progressClock(time_step);
  fromCell(c, s);
  return changed ? 1 : 0;
}

void ref_metabolise(orc_site *s, const orc_params *p) {
  Parameters params = toRef(p);
  Cell c = toCell(s);
  emt6ro::Substrates lv{s->cho, s->ox, s->gi};
  c.metabolise(lv, params.metabolism);
  s->cho = lv.cho; s->ox = lv.ox; s->gi = lv.gi;
}

void ref_irradiate(orc_site *s, float dose, const orc_params *p) {
  Parameters params = toRef(p);
  Cell c = toCell(s);
  c.irradiate(dose, params.cell_repair);
  fromCell(c, s);
}

int ref_try_repair(orc_site *s, const orc_params *p, int cycle_changed, float u, int *used) {
  Parameters params = toRef(p);
  Cell c = toCell(s);
  ReplayRand rr{&u, 1, 0};
  bool alive = c.tryRepair(params.cell_repair, cycle_changed != 0, params.time_step, rr);
  fromCell(c, s);
  *used = rr.i;
  return alive ? 1 : 0;
}

void ref_choose_neighbour_replay(int r, int c, float u, int *rr_out, int *cc_out) {
  ReplayRand rr{&u, 1, 0};
  emt6ro::Coords co = emt6ro::chooseNeighbour(static_cast<uint32_t>(r),
                                              static_cast<uint32_t>(c), rr);
  *rr_out = co.r;
  *cc_out = co.c;
}

void ref_divide_cell_replay(orc_site *parent, orc_site *child, const orc_params *p,
                            const float z[5]) {
  Parameters params = toRef(p);
  Cell pc = toCell(parent);
  ReplayRand rr{z, 5, 0};
  Cell cc = emt6ro::divideCell(pc, params, rr);
  fromCell(pc, parent);
  std::memset(child, 0, sizeof(*child));
  fromCell(cc, child);
}

// ---- file formats through the reference's own loaders ---------------------
int ref_load_params(const char *path, orc_params *out) {
  try {
    Parameters r = Parameters::loadFromJSONFile(path);
    fromRef(r, out);
    return 0;
  } catch (...) {
    return -1;
  }
}

// Writes up to cap sites; returns H*W or -1.
int ref_load_state(const char *path, const orc_params *p, orc_site *out, int cap, int *H,
                   int *W) {
  try {
    Parameters params = toRef(p);
    auto grid = emt6ro::loadFromFile(path, params);
    auto view = grid.view();
    *H = view.dims.height;
    *W = view.dims.width;
    int n = view.dims.vol();
    if (n > cap) return -1;
    for (int k = 0; k < n; ++k) {
      std::memset(&out[k], 0, sizeof(orc_site));
      const Site &s = view.data[k];
      if (s.state == Site::State::OCCUPIED) fromSite(s, &out[k]);
      else {
        out[k].cho = s.substrates.cho;
        out[k].ox = s.substrates.ox;
        out[k].gi = s.substrates.gi;
        out[k].state = static_cast<uint8_t>(s.state);
      }
    }
    return n;
  } catch (...) {
    return -1;
  }
}

// ---- reference CPU path hooks for the ORC_REF_CELL oracle build ------------
void *orc_ref_rng_create(uint32_t seed) { return new emt6ro::HostRandEngine(seed); }
void orc_ref_rng_destroy(void *rng) { delete static_cast<emt6ro::HostRandEngine *>(rng); }

int orc_ref_site_step(orc_site *s, const orc_params *p, uint32_t vac, float dose, void *rng) {
  Parameters params = toRef(p);
  Site site = toSite(s);
  auto &engine = *static_cast<emt6ro::HostRandEngine *>(rng);
  bool ready = site.step(params, static_cast<uint8_t>(vac), dose, engine);
  fromSite(site, s);
  return ready ? 1 : 0;
}

void orc_ref_choose_neighbour(int r, int c, void *rng, int *rr, int *cc) {
  auto &engine = *static_cast<emt6ro::HostRandEngine *>(rng);
  emt6ro::Coords co = emt6ro::chooseNeighbour(static_cast<uint32_t>(r),
                                              static_cast<uint32_t>(c), engine);
  *rr = co.r;
  *cc = co.c;
}

void orc_ref_divide_cell(orc_site *parent, orc_site *child, const orc_params *p, void *rng) {
  Parameters params = toRef(p);
  Cell pc = toCell(parent);
  auto &engine = *static_cast<emt6ro::HostRandEngine *>(rng);
  Cell cc = emt6ro::divideCell(pc, params, engine);
  fromCell(pc, parent);
  std::memset(child, 0, sizeof(*child));
  fromCell(cc, child);
}

}  // extern "C"
