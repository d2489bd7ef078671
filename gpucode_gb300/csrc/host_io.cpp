/*
 * host_io.cpp -- host input/output and set-up derivation of the DEM engine.
 *
 * Replaces the reference's ReadData.cpp, UnitReduce.cpp, DiaInput.cpp,
 * DumpLoad.cpp, WriteTec.cpp and ParticleFeed.cpp, plus the constant
 * derivation inline in main.cpp:328-348 and the scan of IndexOffset.
 *
 * The arithmetic of the set-up (time step, size levels, slot counts, domain,
 * cell sizes, unit reduction, contact constants) follows the reference's
 * expressions operation for operation: cell sizes and grid dimensions feed the
 * cell hash, whose integer output must match the reference exactly.
 *
 * Behavioural differences, by design:
 *  - dem_read_input returns DEM_ERR_IO for a missing file or keyword; the
 *    reference-compatible FindRec/ReadData keep the reference's exit(1).
 *  - DiaInput reads only the numbers present (the reference's feof loop adds
 *    an uninitialised entry when the file ends in whitespace, DiaInput.cpp:22-27)
 *    and never writes past NP entries.
 *  - ParticleFeed draws from a seeded generator (dem_set_feed_seed) instead of
 *    srand(time(NULL)) (ParticleFeed.cpp:17), so feeds are reproducible.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "dem_internal.h"

namespace {

/* heydem.h:15-16 */
constexpr double kPi = 3.1415926;
constexpr double kGravityRef = 9.8f; /* a float literal in the reference */

bool find_key(FILE* f, const char* key) {
  /* ReadData.cpp:7-32: rewind, then the first line whose first strlen(key)
   * characters equal key (a prefix match) */
  char line[260];
  std::rewind(f);
  size_t n = std::strlen(key);
  while (std::fgets(line, 256, f)) {
    if (std::strlen(line) >= n && std::strncmp(line, key, n) == 0) return true;
  }
  return false;
}

bool next_flag_yes(FILE* f) {
  char flag[8] = {0};
  if (!std::fgets(flag, 5, f)) return false;
  return flag[0] == 'Y' || flag[0] == 'y';
}

}  // namespace

/* ---------------------------------------------------------------------- */
/* native input reader                                                      */
/* ---------------------------------------------------------------------- */

extern "C" dem_status dem_read_input(const char* genfile, dem_input* in, double* dia) {
  if (!genfile || !in) return dem::fail(DEM_ERR_ARG, "dem_read_input: null argument");
  std::memset(in, 0, sizeof(*in));
  std::string name = std::string(genfile) + ".in";
  FILE* f = std::fopen(name.c_str(), "rt");
  if (!f) return dem::fail(DEM_ERR_IO, "cannot open " + name);
  auto need = [&](const char* key) -> bool {
    if (find_key(f, key)) return true;
    dem::set_error(std::string("keyword missing in ") + name + ": " + key);
    return false;
  };
  bool ok = true;
  /* main.cpp:65-68 */
  ok = ok && need("NUMPARTICLE") && std::fscanf(f, "%d", &in->np) == 1;
  ok = ok && need("SIZELEVEL") && std::fscanf(f, "%d", &in->n_levels) == 1;
  /* ReadData.cpp:75-187, in the reference's reading order */
  ok = ok && need("LOADMODE") && std::fscanf(f, "%d", &in->load_stage) == 1;
  ok = ok && need("packing_TIME") && std::fscanf(f, "%lf", &in->t_packing) == 1;
  if (ok && need("FoceCapillary")) in->force_cap = next_flag_yes(f) ? 1 : 0; else ok = false;
  ok = ok && need("REALSIZE") && std::fscanf(f, "%lf", &in->real_size) == 1;
  ok = ok && need("CUTGAPFORNEIGHBORLIST") && std::fscanf(f, "%lf", &in->cut_gap) == 1;
  ok = ok && need("EXPANDSIZE") && std::fscanf(f, "%lf", &in->expand_size) == 1;
  if (ok && need("ContainerType")) {
    char bounding[24] = {0};
    if (!std::fgets(bounding, 20, f) || std::strncmp(bounding, "Cylinder", 8) != 0) {
      dem::set_error("ContainerType must be Cylinder");
      ok = false;
    }
  } else {
    ok = false;
  }
  ok = ok && need("CylinderBC") &&
       std::fscanf(f, "%lf %lf %lf %lf %lf", &in->cyl_x, &in->cyl_y, &in->cyl_bw, &in->cyl_r,
                   &in->cyl_h) == 5;
  ok = ok && need("FeedZone") && std::fscanf(f, "%lf %lf", &in->feed_lmin, &in->feed_lmax) == 2;
  if (ok && need("MATERIAL")) {
    for (int m = 0; m < 2 && ok; m++)
      for (int q = 0; q < 7 && ok; q++) ok = std::fscanf(f, "%lf", &in->mat[m][q]) == 1;
  } else {
    ok = false;
  }
  ok = ok && need("LIQUID") && std::fscanf(f, "%lf %lf %lf", &in->lqd[0], &in->lqd[1], &in->lqd[2]) == 3;
  ok = ok && need("SIMULATION") && std::fscanf(f, "%lf %d", &in->dt_factor, &in->n_out) == 2;
  if (ok && need("SIZELEVEL_INPUT")) {
    in->level_input = next_flag_yes(f) ? 1 : 0;
    if (in->level_input) {
      if (in->n_levels < 1 || in->n_levels > DEM_MAX_LEVELS) ok = false;
      for (int i = 0; ok && i < in->n_levels; i++) ok = std::fscanf(f, "%lf", &in->level_dia[i]) == 1;
    }
  } else {
    ok = false;
  }
  std::fclose(f);
  if (!ok) {
    if (dem::last_error_empty()) dem::set_error("parse error in " + name);
    return DEM_ERR_IO;
  }
  if (in->np <= 0 || in->n_levels < 1 || in->n_levels > DEM_MAX_LEVELS)
    return dem::fail(DEM_ERR_IO, "NUMPARTICLE / SIZELEVEL out of range in " + name);
  if (!dia) return DEM_OK;
  /* ReadData.cpp:216-235: <genfile>_dia.dat if present, else REALSIZE for all */
  std::string dname = std::string(genfile) + "_dia.dat";
  FILE* df = std::fopen(dname.c_str(), "rt");
  if (df) {
    std::fclose(df);
    std::vector<double> rad(in->np);
    dem_status st = dem::read_diameters(dname.c_str(), rad.data(), in->np);
    if (st != DEM_OK) return st;
    for (int i = 0; i < in->np; i++) dia[i] = rad[i] * 2.0;
  } else {
    for (int i = 0; i < in->np; i++) dia[i] = in->real_size;
  }
  return DEM_OK;
}

namespace dem {

/* DiaInput.cpp:8-49, reading only what is there: diameters after the
 * "PARTICLE DIAMETER" line, tiled cyclically over np particles, halved. */
dem_status read_diameters(const char* path, double* hRad, int np) {
  FILE* f = std::fopen(path, "rt");
  if (!f) return fail(DEM_ERR_IO, std::string("cannot open ") + path);
  if (!find_key(f, "PARTICLE DIAMETER")) {
    std::fclose(f);
    return fail(DEM_ERR_IO, std::string("keyword PARTICLE DIAMETER missing in ") + path);
  }
  std::vector<double> d;
  double v;
  while ((int)d.size() < np && std::fscanf(f, "%lf", &v) == 1) d.push_back(v);
  std::fclose(f);
  if (d.empty()) return fail(DEM_ERR_IO, std::string("no diameters in ") + path);
  for (int k = 0; k < np; k++) hRad[k] = d[k % d.size()] / 2.0f;
  return DEM_OK;
}

}  // namespace dem

/* ---------------------------------------------------------------------- */
/* set-up derivation                                                        */
/* ---------------------------------------------------------------------- */

namespace {

/* ReadData.cpp:165-166 + 243-375 (real units); fills everything but the unit
 * reduction.  Returns false on an inconsistent input. */
bool derive_real(const dem_input* in, const double* dia, dem_setup* s, double* hRad, int* pLevel,
                 int* neborIdx, double* cutGap_out) {
  const int NP = in->np, nL = in->n_levels;
  for (int m = 0; m < 2; m++) {
    MatType& M = s->mat[m];
    M.density = in->mat[m][0];
    M.ymod = in->mat[m][1];
    M.pois = in->mat[m][2];
    M.sfrc = in->mat[m][3];
    M.rfrc = in->mat[m][4];
    M.dmpn = in->mat[m][5];
    M.yldp = in->mat[m][6];
    M.emod = M.ymod / (1 - M.pois * M.pois);
  }
  s->lqd.stension = in->lqd[0];
  s->lqd.vol = in->lqd[1];
  s->lqd.gapmn = in->lqd[2];
  s->lqd.layer = 0.0;
  s->lqd.brknmx = 0.0;
  s->cyl.cir.x = in->cyl_x;
  s->cyl.cir.y = in->cyl_y;
  s->cyl.Bw = in->cyl_bw;
  s->cyl.R = in->cyl_r;
  s->cyl.Tw = in->cyl_bw + in->cyl_h;
  s->cyl.topv = 0.0;
  s->cyl.btmv = 0.0;
  s->feed.Lmin = in->feed_lmin;
  s->feed.Lmax = in->feed_lmax;
  s->force_cap = in->force_cap;
  s->load.stage = in->load_stage;
  s->load.tPacking = in->t_packing;
  s->load.nOutPacking = in->n_out;
  s->load_stage = in->load_stage;
  s->init_par_size = in->real_size;
  for (int i = 0; i < NP; i++) hRad[i] = dia[i] / 2.0f;
  /* time step, ReadData.cpp:243-263 */
  const double e0 = s->mat[0].emod;
  double pwemod = 2.0f * e0 * e0 / (e0 + e0);
  double rmin = hRad[0], rmax = hRad[0];
  for (int i = 1; i < NP; i++) {
    if (hRad[i] <= rmin) rmin = hRad[i];
    if (hRad[i] >= rmax) rmax = hRad[i];
  }
  double sizeMn = 2.0 * rmin;
  double stiffk = 1.333 * pwemod * std::sqrt(sizeMn * 0.25);
  double massMn = s->mat[0].density * kPi * std::pow(sizeMn, 3.0) / 6.0;
  s->sim.dtFactor = in->dt_factor;
  s->sim.dt = in->dt_factor * kPi * std::sqrt(0.5 * massMn / stiffk) * std::pow(10.0, -0.2);
  if (in->dt_override > 0.0) s->sim.dt = in->dt_override;
  s->sim.cutGap = in->cut_gap;
  /* size levels, ReadData.cpp:273-293 */
  if (in->level_input) {
    for (int i = 0; i < nL; i++) s->level_size[i] = in->level_dia[i] / 2;
  } else {
    double gap = (rmax - rmin) / nL;
    for (int i = 0; i < nL; i++) s->level_size[i] = gap * (i + 1) + rmin;
  }
  /* slots per level, ReadData.cpp:299-307 */
  for (int i = 0; i < nL; i++) {
    double S = s->level_size[i] / rmin;
    s->level_nnebors[i] =
        (int)std::ceil(1.2 * (std::pow((S + 2 + s->sim.cutGap), 3.0) - std::pow(S, 3.0)));
    s->level_npars[i] = 0;
  }
  /* particle -> level and rank within the level, ReadData.cpp:311-334 */
  for (int i = 0; i < NP; i++) {
    pLevel[i] = -1;
    neborIdx[i] = 0;
    if (hRad[i] <= s->level_size[0]) {
      pLevel[i] = 0;
      neborIdx[i] = s->level_npars[0]++;
    } else {
      for (int L = 1; L < nL; L++) {
        if (hRad[i] > s->level_size[L - 1] && hRad[i] <= s->level_size[L]) {
          pLevel[i] = L;
          neborIdx[i] = s->level_npars[L]++;
        }
      }
    }
    if (pLevel[i] < 0) {
      dem::set_error("particle " + std::to_string(i) + " fits no size level");
      return false;
    }
  }
  /* computing zone, ReadData.cpp:136-137, 350-357 */
  double ex = in->expand_size * rmax;
  s->prm.Origin.x = (s->cyl.cir.x - s->cyl.R) - ex;
  s->prm.Origin.y = (s->cyl.cir.y - s->cyl.R) - ex;
  s->prm.Origin.z = s->cyl.Bw - ex;
  s->prm.EndPoint.x = (s->cyl.cir.x + s->cyl.R) + ex;
  s->prm.EndPoint.y = (s->cyl.cir.y + s->cyl.R) + ex;
  s->prm.EndPoint.z = s->cyl.Tw + ex;
  /* ReadData.cpp:363-375 */
  s->sim.cutGap = s->sim.cutGap * (rmin / rmax);
  long long total = 0;
  for (int i = 0; i < nL; i++) {
    s->cell_size[i] = (1.0 + s->sim.cutGap * 1.4) * 2.0 * s->level_size[i];
    s->grid_size[i].x = (int)std::ceil((s->prm.EndPoint.x - s->prm.Origin.x) / s->cell_size[i]);
    s->grid_size[i].y = (int)std::ceil((s->prm.EndPoint.y - s->prm.Origin.y) / s->cell_size[i]);
    s->grid_size[i].z = (int)std::ceil((s->prm.EndPoint.z - s->prm.Origin.z) / s->cell_size[i]);
    long long nc = (long long)s->grid_size[i].x * s->grid_size[i].y * s->grid_size[i].z;
    if (nc <= 0 || nc > 0x7fffffffLL) {
      dem::set_error("cell grid of level " + std::to_string(i) + " out of int range");
      return false;
    }
    s->num_cells[i] = (int)nc;
    total += nc;
  }
  if (total > 0x7fffffffLL) {
    dem::set_error("total cell count out of int range");
    return false;
  }
  *cutGap_out = s->sim.cutGap;
  s->rad_min = rmin;
  s->rad_max = rmax;
  return true;
}

}  // namespace

namespace dem {

/* UnitReduce.cpp:14-104 on the set-up struct (the same arithmetic as the
 * exported UnitReduce below). */
void unit_reduce(dem_setup* s, double* hRad, int np, double gravity) {
  UNIT& U = s->unit;
  const double D = s->init_par_size;
  U.rlunit = D;
  U.rmunit = s->mat[0].density * kPi * std::pow(D, 3.0) / 6.0;
  U.rfunit = U.rmunit * gravity;
  U.rsunit = U.rfunit / std::pow(D, 2.0);
  U.rtunit = std::pow(D / gravity, 0.5);
  U.rvunit = U.rlunit / U.rtunit;
  U.reunit = U.rmunit * gravity * U.rlunit;
  s->cyl.cir.x = s->cyl.cir.x / U.rlunit;
  s->cyl.cir.y = s->cyl.cir.y / U.rlunit;
  s->cyl.Tw = s->cyl.Tw / U.rlunit;
  s->cyl.Bw = s->cyl.Bw / U.rlunit;
  s->cyl.R = s->cyl.R / U.rlunit;
  for (int i = 0; i < s->n_levels; i++) s->level_size[i] = s->level_size[i] / U.rlunit;
  s->feed.Lmax = s->feed.Lmax / U.rlunit;
  s->feed.Lmin = s->feed.Lmin / U.rlunit;
  s->load.tPacking = s->load.tPacking / U.rtunit;
  for (int k = 0; k < np; k++) hRad[k] = hRad[k] / U.rlunit;
  for (int m = 0; m < 2; m++) {
    s->mat[m].emod = s->mat[m].emod * std::pow(U.rlunit, 2.0) / U.rfunit;
    s->mat[m].yldp = s->mat[m].yldp * std::pow(U.rlunit, 2.0) / U.rfunit;
    s->mat[m].dmpn = s->mat[m].dmpn / U.rtunit;
  }
  LIQUID& L = s->lqd;
  L.gapmn = L.gapmn / D;
  L.layer = 0.5 * (std::pow((1.0 + L.vol), 1.0 / 3.0) - 1.0);
  L.vol = L.vol * kPi / 6.0;
  L.stension = L.stension * U.rlunit / U.rfunit;
  L.brknmx = 0.99 * std::pow((L.vol / 6.0), 0.34);
  s->sim.dt = s->sim.dt / U.rtunit;
  s->sim.outtime = s->sim.outtime / U.rtunit;
  s->sim.outinterval = s->sim.outinterval / U.rtunit;
  s->sim.fdinterval = s->sim.fdinterval / U.rtunit;
  s->prm.Origin.x = s->prm.Origin.x / U.rlunit;
  s->prm.Origin.y = s->prm.Origin.y / U.rlunit;
  s->prm.Origin.z = s->prm.Origin.z / U.rlunit;
  s->prm.EndPoint.x = s->prm.EndPoint.x / U.rlunit;
  s->prm.EndPoint.y = s->prm.EndPoint.y / U.rlunit;
  s->prm.EndPoint.z = s->prm.EndPoint.z / U.rlunit;
  for (int i = 0; i < s->n_levels; i++) s->cell_size[i] = s->cell_size[i] / U.rlunit;
  s->prm.dt = s->sim.dt;
  s->prm.NP = np;
  s->prm.SearchGap = s->sim.cutGap;
}

/* main.cpp:328-348 */
void derive_contact_constants(dem_setup* s) {
  const MatType* M = s->mat;
  calParaPP& c = s->cal;
  std::memset(&c, 0, sizeof(c));
  c.emod = (M[0].emod * M[0].emod) / (M[0].emod + M[0].emod);
  c.pois = 2.0 * (M[0].pois * M[0].pois) / (M[0].pois + M[0].pois);
  c.sfrc = M[0].sfrc;
  c.ystress = M[0].yldp * M[0].yldp / (M[0].yldp + M[0].yldp);
  c.ydsp_t = std::pow((kPi * c.ystress / (2.0 * c.emod)), 2.0);
  c.yforce_t = 4.0 / 3.0 * c.emod * std::pow(c.ydsp_t, 1.5);
  c.ystiff_t = kPi * c.ystress;
  calParaPW& w = s->pwcal;
  std::memset(&w, 0, sizeof(w));
  w.emod = M[0].emod;
  w.pois = 2.0 * (M[0].pois * M[1].pois) / (M[0].pois + M[1].pois);
  w.sfrc = std::pow(M[1].sfrc * M[1].sfrc, 0.5);
  w.ystress = M[0].yldp;
  w.ydsp_t = std::pow((kPi * w.ystress / (2.0 * w.emod)), 2.0);
  w.yforce_t = 4.0 / 3.0 * w.emod * std::pow(w.ydsp_t, 1.5);
  w.ystiff_t = kPi * w.ystress;
}

}  // namespace dem

extern "C" dem_status dem_build_setup(const dem_input* in, const double* dia, dem_setup* s,
                                      double* rad, int* plevel, int* nebor_idx) {
  if (!in || !dia || !s || !rad || !plevel || !nebor_idx)
    return dem::fail(DEM_ERR_ARG, "dem_build_setup: null argument");
  if (in->np <= 0 || in->n_levels < 1 || in->n_levels > DEM_MAX_LEVELS)
    return dem::fail(DEM_ERR_ARG, "dem_build_setup: np / n_levels out of range");
  std::memset(s, 0, sizeof(*s));
  s->np = in->np;
  s->n_levels = in->n_levels;
  double cutGap = 0.0;
  if (!derive_real(in, dia, s, rad, plevel, nebor_idx, &cutGap)) return DEM_ERR_ARG;
  const double g = in->gravity > 0.0 ? in->gravity : kGravityRef;
  dem::unit_reduce(s, rad, in->np, g);
  s->rad_min = s->rad_min / s->unit.rlunit;
  s->rad_max = s->rad_max / s->unit.rlunit;
  dem::derive_contact_constants(s);
  /* IndexOffset (ParticleSystem.cu:72-77): inclusive scan of cell counts */
  int acc = 0;
  for (int i = 0; i < s->n_levels; i++) {
    acc += s->num_cells[i];
    s->ncell_idx[i] = acc;
  }
  s->sys_ncells = acc;
  long long slots = 0;
  for (int i = 0; i < s->n_levels; i++) slots += (long long)s->level_npars[i] * s->level_nnebors[i];
  s->n_pp_slots = slots;
  /* main.cpp:401-403 */
  s->sim.simTime = s->load.tPacking;
  s->sim.outinterval = s->load.nOutPacking > 0 ? s->sim.simTime / s->load.nOutPacking : 0.0;
  s->sim.fdinterval = 1.0 * s->sim.outinterval;
  return DEM_OK;
}

/* ---------------------------------------------------------------------- */
/* reference-compatible host functions (heydem.h:407-441)                    */
/* ---------------------------------------------------------------------- */

extern "C" void FindRec(FILE* inFile, char* strDest) {
  /* ReadData.cpp:7-32: a missing key ends the program with exit(1) */
  if (!inFile || !strDest || !find_key(inFile, strDest)) std::exit(1);
}

extern "C" void DiaInput(char* diaFile, double* hRad, int NP) {
  if (dem::read_diameters(diaFile, hRad, NP) != DEM_OK) {
    std::fprintf(stderr, "DiaInput: %s\n", dem_last_error());
    std::exit(1);
  }
}

extern "C" void LoadPara(char* DumpName, int* NP, int* nBatch, int* TotalParticle) {
  /* DumpLoad.cpp:7-19: three integers after the "SYSTEM Info" line */
  FILE* f = std::fopen(DumpName, "rt");
  if (!f) std::exit(1);
  FindRec(f, (char*)"SYSTEM Info");
  if (std::fscanf(f, "%d %d %d", NP, nBatch, TotalParticle) != 3) std::exit(1);
  std::fclose(f);
}

extern "C" void ReadData(double* h_Level_size, int* h_pLevel, int* h_level_nNebors,
                         int* h_level_nPars, int* h_Nebor_Idx, CylinderBC** h_Cir,
                         CylinderBC** d_Cir, FeedZone* Feedcube, MatType* h_Mat, LIQUID* h_lqd,
                         PARAMETER* h_Params, double* InitParSize, int* ForceCap,
                         SIMULATION* h_dem, LOADMODE* h_load, double* hRad, SEARCHCELL h_cell,
                         int NP, int nLevels, char* genfile, int RESTART) {
  (void)RESTART;
  dem_input in;
  std::vector<double> dia((size_t)NP);
  if (dem_read_input(genfile, &in, dia.data()) != DEM_OK) {
    std::fprintf(stderr, "ReadData: %s\n", dem_last_error());
    std::exit(1);
  }
  in.np = NP;
  in.n_levels = nLevels;
  dem_setup s;
  std::memset(&s, 0, sizeof(s));
  s.np = NP;
  s.n_levels = nLevels;
  double cutGap = 0.0;
  if (!derive_real(&in, dia.data(), &s, hRad, h_pLevel, h_Nebor_Idx, &cutGap)) {
    std::fprintf(stderr, "ReadData: %s\n", dem_last_error());
    std::exit(1);
  }
  /* outputs in real units, as the reference leaves them for UnitReduce */
  for (int i = 0; i < nLevels; i++) {
    h_Level_size[i] = s.level_size[i];
    h_level_nNebors[i] = s.level_nnebors[i];
    h_level_nPars[i] = s.level_npars[i];
    h_cell.Cellsize[i] = s.cell_size[i];
    h_cell.gridSize[i] = s.grid_size[i];
    h_cell.numCells[i] = s.num_cells[i];
  }
  *h_Cir = (CylinderBC*)std::malloc(sizeof(CylinderBC));
  **h_Cir = s.cyl;
  if (dem::cuda_alloc((void**)d_Cir, sizeof(CylinderBC)) != DEM_OK) std::exit(-1);
  *Feedcube = s.feed;
  h_Mat[0] = s.mat[0];
  h_Mat[1] = s.mat[1];
  *h_lqd = s.lqd;
  h_Params->Origin = s.prm.Origin;
  h_Params->EndPoint = s.prm.EndPoint;
  *InitParSize = s.init_par_size;
  *ForceCap = in.force_cap ? 1 : *ForceCap;
  /* ReadData.cpp:186-199 */
  h_dem->dtFactor = in.dt_factor;
  h_dem->simTime = 0.0;
  h_dem->dumptime = 0.0;
  h_dem->outtime = 0.0;
  h_dem->ctime = 0.0;
  h_dem->iter = 0;
  h_dem->fdtime = 0.0;
  h_dem->Outs = 0;
  h_dem->dt = s.sim.dt;
  h_dem->cutGap = cutGap;
  h_load->stage = in.load_stage;
  h_load->tPacking = in.t_packing;
  h_load->nOutPacking = in.n_out;
}

extern "C" void UnitReduce(UNIT* Rdu, CylinderBC* h_Cir, FeedZone* Feedcube, LOADMODE* h_load,
                           double* hRad, MatType* h_Mat, LIQUID* h_lqd, double InitParSize,
                           SIMULATION* h_dem, PARAMETER* h_Params, SEARCHCELL h_cell,
                           double* h_Level_size, int nLevels, int NP, int RESTART, char* genfile) {
  (void)RESTART;
  (void)genfile;
  dem_setup s;
  std::memset(&s, 0, sizeof(s));
  s.n_levels = nLevels;
  s.init_par_size = InitParSize;
  s.cyl = *h_Cir;
  s.feed = *Feedcube;
  s.load = *h_load;
  s.mat[0] = h_Mat[0];
  s.mat[1] = h_Mat[1];
  s.lqd = *h_lqd;
  s.sim = *h_dem;
  s.prm = *h_Params;
  for (int i = 0; i < nLevels; i++) {
    s.level_size[i] = h_Level_size[i];
    s.cell_size[i] = h_cell.Cellsize[i];
  }
  dem::unit_reduce(&s, hRad, NP, kGravityRef);
  *Rdu = s.unit;
  *h_Cir = s.cyl;
  *Feedcube = s.feed;
  *h_load = s.load;
  h_Mat[0] = s.mat[0];
  h_Mat[1] = s.mat[1];
  *h_lqd = s.lqd;
  *h_dem = s.sim;
  *h_Params = s.prm;
  for (int i = 0; i < nLevels; i++) {
    h_Level_size[i] = s.level_size[i];
    h_cell.Cellsize[i] = s.cell_size[i];
  }
}

extern "C" void WrtTec(double3* hPos, double3* hVel, double3* hForce, double3* hAngVel,
                       SIMULATION* h_dem, double* hRad, UNIT* Rdu, int TotalParticle, int NP) {
  (void)NP;
  /* WriteTec.cpp:9-38: header on the first output, then one zone per call */
  const char* filename = "particle_info.dat";
  if (h_dem->Outs == 0) {
    FILE* o = std::fopen(filename, "wt");
    if (!o) return;
    std::fprintf(o, "TITLE = \" PARTICLE INFORMATION \" \n");
    std::fprintf(o, "VARIABLES = X   Y   Z   R   VX   VY   VZ   W   F\n");
    std::fclose(o);
  }
  FILE* o = std::fopen(filename, "a");
  if (!o) return;
  std::fprintf(o, "ZONE T= \" %12.6lf s \" \n", h_dem->ctime * Rdu->rtunit);
  for (int ip = 0; ip < TotalParticle; ip++) {
    const double3 w = hAngVel[ip], F = hForce[ip];
    std::fprintf(o,
                 "%11.5lf   %11.5lf   %11.5lf   %11.5f  %11.5lf   %11.5lf   %11.5lf   %11.5lf   "
                 "%11.5lf\n",
                 hPos[ip].x, hPos[ip].y, hPos[ip].z, hRad[ip], hVel[ip].x, hVel[ip].y, hVel[ip].z,
                 std::sqrt(w.x * w.x + w.y * w.y + w.z * w.z),
                 std::sqrt(F.x * F.x + F.y * F.y + F.z * F.z));
  }
  std::fclose(o);
}

/* ---------------------------------------------------------------------- */
/* binary column output beside WrtTec                                       */
/* ---------------------------------------------------------------------- */

extern "C" void WrtBin(double3* hPos, double3* hVel, double3* hForce, double3* hAngVel, SIMULATION* h_dem,
                       double* hRad, UNIT* Rdu, int TotalParticle, int NP) {
  (void)NP;
  /* WrtTec's quantities (WriteTec.cpp:28-35) at full precision, one column
   * after the other: a file header on the first output (magic, column count,
   * eight-byte column names), then per call a zone: tag, time [s], count and
   * the nine columns of `count` doubles */
  const char* filename = "particle_info.bin";
  static const char names[9][8] = {"X", "Y", "Z", "R", "VX", "VY", "VZ", "W", "F"};
  if (h_dem->Outs == 0) {
    FILE* o = std::fopen(filename, "wb");
    if (!o) return;
    const char magic[8] = {'D', 'E', 'M', 'C', 'O', 'L', '0', '1'};
    const int ncol = 9;
    std::fwrite(magic, 1, 8, o);
    std::fwrite(&ncol, sizeof(int), 1, o);
    std::fwrite(names, 8, 9, o);
    std::fclose(o);
  }
  FILE* o = std::fopen(filename, "ab");
  if (!o) return;
  const char tag[8] = {'Z', 'O', 'N', 'E', 0, 0, 0, 0};
  const double t = h_dem->ctime * Rdu->rtunit;
  const long long n = TotalParticle > 0 ? TotalParticle : 0;
  std::fwrite(tag, 1, 8, o);
  std::fwrite(&t, sizeof(double), 1, o);
  std::fwrite(&n, sizeof(long long), 1, o);
  std::vector<double> buf((size_t)std::min<long long>(n, 1 << 16));
  for (int col = 0; col < 9; col++) {
    for (long long i0 = 0; i0 < n; i0 += (long long)buf.size()) {
      const long long m = std::min<long long>((long long)buf.size(), n - i0);
      for (long long k = 0; k < m; k++) {
        const long long ip = i0 + k;
        double v;
        switch (col) {
          case 0: v = hPos[ip].x; break;
          case 1: v = hPos[ip].y; break;
          case 2: v = hPos[ip].z; break;
          case 3: v = hRad[ip]; break;
          case 4: v = hVel[ip].x; break;
          case 5: v = hVel[ip].y; break;
          case 6: v = hVel[ip].z; break;
          case 7: {
            const double3 w = hAngVel[ip];
            v = std::sqrt(w.x * w.x + w.y * w.y + w.z * w.z);
            break;
          }
          default: {
            const double3 F = hForce[ip];
            v = std::sqrt(F.x * F.x + F.y * F.y + F.z * F.z);
          }
        }
        buf[(size_t)k] = v;
      }
      std::fwrite(buf.data(), sizeof(double), (size_t)m, o);
    }
  }
  std::fclose(o);
}

/* ---------------------------------------------------------------------- */
/* seeded feed (ParticleFeed.cpp:8-72)                                      */
/* ---------------------------------------------------------------------- */

namespace {
uint64_t g_feed_state = 0x9E3779B97F4A7C15ull;

/* SplitMix64 (Steele, Lea, Flood 2014) -> uniform double in [0, 1] */
double feed_uniform() {
  uint64_t z = (g_feed_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740991.0);
}
}  // namespace

extern "C" void dem_set_feed_seed(unsigned long long seed) { g_feed_state = seed; }

extern "C" int ParticleFeed(FeedZone* Feedcube, CylinderBC* h_Cir, double InitParSize,
                            double3* hPos, double* hRad, int numParticle, int NP) {
  (void)InitParSize;
  /* Rejection sampling in the disc x [Lmin, Lmax] band with a 0.002 clearance:
   * up to 60000 placements per call, giving up after 500 consecutive
   * rejections.  The overlap test uses a uniform bucket grid instead of the
   * reference's scan over every placed particle; the accepted set is the same
   * for the same random stream. */
  const double zmin = Feedcube->Lmin, zmax = Feedcube->Lmax;
  const double clear = 0.002;
  double rmax = 0.0;
  for (int i = 0; i < NP; i++) rmax = hRad[i] > rmax ? hRad[i] : rmax;
  const double cell = 2.0 * rmax + clear > 0.0 ? 2.0 * rmax + clear : 1.0;
  const double x0 = h_Cir->cir.x - h_Cir->R, y0 = h_Cir->cir.y - h_Cir->R;
  double zlo = zmin, zhi = zmax;
  for (int i = 0; i < numParticle; i++) {
    zlo = hPos[i].z < zlo ? hPos[i].z : zlo;
    zhi = hPos[i].z > zhi ? hPos[i].z : zhi;
  }
  const int gx = (int)std::ceil(2.0 * h_Cir->R / cell) + 1;
  const int gz = (int)std::ceil((zhi - zlo) / cell) + 1;
  const long long ncell = (long long)gx * gx * gz;
  std::vector<std::vector<int>> bucket((size_t)(ncell > 0 && ncell < 50000000 ? ncell : 1));
  const bool use_grid = ncell > 0 && ncell < 50000000;
  auto key = [&](double3 p) -> long long {
    int ix = (int)std::floor((p.x - x0) / cell), iy = (int)std::floor((p.y - y0) / cell);
    int iz = (int)std::floor((p.z - zlo) / cell);
    ix = ix < 0 ? 0 : (ix >= gx ? gx - 1 : ix);
    iy = iy < 0 ? 0 : (iy >= gx ? gx - 1 : iy);
    iz = iz < 0 ? 0 : (iz >= gz ? gz - 1 : iz);
    return ((long long)iz * gx + iy) * gx + ix;
  };
  if (use_grid)
    for (int i = 0; i < numParticle; i++) bucket[(size_t)key(hPos[i])].push_back(i);
  int nEach = 0, misses = 0;
  while (misses < 500 && numParticle < NP && nEach < 60000) {
    double theta = 2.0 * kPi * feed_uniform();
    double u = feed_uniform() + feed_uniform();
    double mag = u > 1 ? 2 - u : u;
    double3 p;
    p.x = mag * (h_Cir->R - hRad[numParticle]) * std::cos(theta) + h_Cir->cir.x;
    p.y = mag * (h_Cir->R - hRad[numParticle]) * std::sin(theta) + h_Cir->cir.y;
    p.z = feed_uniform() * (zmax - zmin) + zmin;
    bool overlap = false;
    auto test = [&](int i) {
      double dx = p.x - hPos[i].x, dy = p.y - hPos[i].y, dz = p.z - hPos[i].z;
      return std::sqrt(dx * dx + dy * dy + dz * dz) < (hRad[i] + hRad[numParticle] + clear);
    };
    if (use_grid) {
      long long k = key(p);
      int kx = (int)(k % gx), ky = (int)((k / gx) % gx), kz = (int)(k / ((long long)gx * gx));
      for (int dz = -1; dz <= 1 && !overlap; dz++)
        for (int dy = -1; dy <= 1 && !overlap; dy++)
          for (int dx = -1; dx <= 1 && !overlap; dx++) {
            int x = kx + dx, y = ky + dy, z = kz + dz;
            if (x < 0 || y < 0 || z < 0 || x >= gx || y >= gx || z >= gz) continue;
            for (int i : bucket[((size_t)z * gx + y) * gx + x])
              if (test(i)) { overlap = true; break; }
          }
    } else {
      for (int i = 0; i < numParticle && !overlap; i++) overlap = test(i);
    }
    if (overlap) {
      misses++;
      continue;
    }
    hPos[numParticle] = p;
    if (use_grid) bucket[(size_t)key(p)].push_back(numParticle);
    numParticle++;
    nEach++;
    misses = 0;
  }
  return numParticle;
}

/* ---------------------------------------------------------------------- */
/* seeded deposition packer (benchmark and test inputs)                     */
/* ---------------------------------------------------------------------- */

extern "C" dem_status dem_scale_cells(dem_setup* s, double factor) {
  if (!s || !(factor >= 1.0) || factor > 16.0) return dem::fail(DEM_ERR_ARG, "dem_scale_cells: factor must be in [1, 16]");
  if (factor == 1.0) return DEM_OK;
  /* larger cells keep every pair within one cell of each other, so the
   * neighbour search (the 27 surrounding cells of each level) stays complete */
  dem_setup t = *s;
  long long total = 0;
  for (int i = 0; i < t.n_levels; i++) {
    t.cell_size[i] *= factor;
    t.grid_size[i].x = (int)std::ceil((t.prm.EndPoint.x - t.prm.Origin.x) / t.cell_size[i]);
    t.grid_size[i].y = (int)std::ceil((t.prm.EndPoint.y - t.prm.Origin.y) / t.cell_size[i]);
    t.grid_size[i].z = (int)std::ceil((t.prm.EndPoint.z - t.prm.Origin.z) / t.cell_size[i]);
    const long long nc = (long long)t.grid_size[i].x * t.grid_size[i].y * t.grid_size[i].z;
    if (nc <= 0) return dem::fail(DEM_ERR_ARG, "dem_scale_cells: empty grid");
    t.num_cells[i] = (int)nc;
    total += nc;
    t.ncell_idx[i] = (int)total;
  }
  t.sys_ncells = (int)total;
  *s = t;
  return DEM_OK;
}

extern "C" dem_status dem_pack_deposit(int n, const double* dia, double cx, double cy, double R, double z0,
                                       double gap, int tries, unsigned long long seed, double3* pos_out) {
  if (n <= 0 || !dia || !pos_out || R <= 0.0 || tries < 1)
    return dem::fail(DEM_ERR_ARG, "dem_pack_deposit: bad argument");
  double dmax = 0.0;
  for (int i = 0; i < n; i++) dmax = dia[i] > dmax ? dia[i] : dmax;
  if (!(dmax > 0.0) || 2.0 * R <= dmax) return dem::fail(DEM_ERR_ARG, "dem_pack_deposit: particles do not fit");
  /* 2-D buckets over the disc; each keeps its spheres sorted by the height of
   * their tops, so a falling sphere scans a bucket from the top down and stops
   * as soon as no lower sphere could be reached (exact, no pruning) */
  const double cell = dmax + gap;
  const int g = (int)std::ceil(2.0 * R / cell) + 1;
  const double x0 = cx - R, y0 = cy - R;
  std::vector<std::vector<int>> bucket((size_t)g * g);
  uint64_t st = seed ? seed : 0x2545F4914F6CDD1Dull;
  auto uni = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  auto top_of = [&](int j) { return pos_out[j].z + 0.5 * dia[j]; };
  for (int i = 0; i < n; i++) {
    const double ri = 0.5 * dia[i];
    const double rr = R - ri - gap;
    if (rr <= 0.0) return dem::fail(DEM_ERR_ARG, "dem_pack_deposit: particle wider than the cylinder");
    double best_z = 1e300, bx = cx, by = cy;
    for (int t = 0; t < tries; t++) {
      const double th = 2.0 * kPi * uni();
      const double rad = rr * std::sqrt(uni());
      const double x = cx + rad * std::cos(th), y = cy + rad * std::sin(th);
      double z = z0 + ri + gap;
      const int ix = (int)((x - x0) / cell), iy = (int)((y - y0) / cell);
      /* the 9 buckets around the drop point, walked together from the highest
       * top down: the first spheres met are the ones the drop lands on, and
       * the walk ends when the next top is too low to raise the landing
       * height (each bucket alone would be scanned to the floor whenever the
       * drop misses its upper spheres) */
      const std::vector<int>* B[9];
      size_t head[9];
      int nb = 0;
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const int bxi = ix + dx, byi = iy + dy;
          if (bxi < 0 || byi < 0 || bxi >= g || byi >= g) continue;
          const std::vector<int>& L = bucket[(size_t)byi * g + bxi];
          if (L.empty()) continue;
          B[nb] = &L;
          head[nb] = L.size();
          nb++;
        }
      for (;;) {
        int pick = -1;
        double best_top = -1e300;
        for (int b = 0; b < nb; b++) {
          if (head[b] == 0) continue;
          const double t = top_of((*B[b])[head[b] - 1]);
          if (t > best_top) {
            best_top = t;
            pick = b;
          }
        }
        /* the highest landing height sphere j can give is its top + ri + gap */
        if (pick < 0 || best_top + ri + gap <= z) break;
        const int j = (*B[pick])[--head[pick]];
        const double reach = ri + 0.5 * dia[j] + gap;
        const double hx = x - pos_out[j].x, hy = y - pos_out[j].y;
        const double h2 = hx * hx + hy * hy;
        if (h2 >= reach * reach) continue;
        const double zc = pos_out[j].z + std::sqrt(reach * reach - h2);
        if (zc > z) z = zc;
      }
      if (z < best_z) {
        best_z = z;
        bx = x;
        by = y;
      }
    }
    pos_out[i].x = bx;
    pos_out[i].y = by;
    pos_out[i].z = best_z;
    const int ix = (int)((bx - x0) / cell), iy = (int)((by - y0) / cell);
    std::vector<int>& L = bucket[(size_t)iy * g + ix];
    /* insert keeping tops ascending (new spheres land near the top) */
    L.push_back(i);
    for (size_t r = L.size() - 1; r > 0 && top_of(L[r - 1]) > top_of(L[r]); r--) std::swap(L[r - 1], L[r]);
  }
  return DEM_OK;
}
