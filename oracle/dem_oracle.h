/*
 * dem_oracle.h -- CPU oracle for the per-step DEM path (TEST INFRASTRUCTURE).
 *
 * A plain-C, FP64 restatement of the reference heyDEM step (cell hash -> sort ->
 * cell start/end -> neighbour lists -> contact-history carry-over -> wall list ->
 * p-p contact + capillary -> cylinder-wall contact -> integrator), in the
 * reference's own data layouts (AoS double3, level/slot-major neighbour slots,
 * slot-major history, [particle][3] wall list).  Each function cites the
 * reference file:line it restates.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
 * library, and only as the checker / the timed CPU baseline.  The product path
 * (libdem_gb300) never links or calls it.
 *
 * Parity pin: tests/test_oracle_pin.py runs every function here against the
 * reference's own kernel.cu compiled for the CPU (oracle/_ref, built by
 * oracle/build_ref.sh from the reference sources in place) on seeded inputs and
 * requires bit-identical results; tests/golden/ holds fixtures generated from
 * that build so the pin also holds where the reference sources are absent.
 *
 * Struct layouts match the reference's heydem.h (including double2's 16-byte
 * alignment inside CylinderBC) so the same buffers can be handed to either side.
 */
#ifndef DEM_ORACLE_H
#define DEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#ifdef __cplusplus
#define ORC_ALIGN16 alignas(16)
#else
#define ORC_ALIGN16 _Alignas(16)
#endif

typedef struct { double x, y, z; } ov3; /* CUDA double3 */
typedef struct { int x, y, z; } oi3;    /* CUDA int3 */

/* heydem.h:39-46 CylinderBC (double2 cir is 16-byte aligned) */
typedef struct {
  ORC_ALIGN16 double cir_x;
  double cir_y;
  double R, Tw, Bw, topv, btmv;
} o_cylinder;

/* heydem.h:90-97 MatType */
typedef struct { double density, emod, ymod, pois, dmpn, sfrc, rfrc, yldp; } o_mat;
/* heydem.h:104-111 LIQUID */
typedef struct { double stension, vol, gapmn, layer, brknmx; } o_liquid;
/* heydem.h:196-204 PARAMETER */
typedef struct { ov3 Origin; ov3 EndPoint; double SearchGap; double dt; int NP; } o_parameter;
/* heydem.h:220-229 calParaPP (calParaPW has the same layout, heydem.h:233-242) */
typedef struct { double emod, pois, sfrc, ystress, ydsp_t, yforce_t, ystiff_t; } o_calpara;

/* the constant-memory set of kernel.cu:15-19, then this library's per-contact
 * liquid model (no counterpart in the reference: lqd_mode 0 is the reference's
 * model and the reference's own kernels never read these fields) */
typedef struct {
  o_mat mat[2];
  o_liquid lqd;
  o_parameter prm;
  o_calpara cal;   /* p-p */
  o_calpara pwcal; /* p-wall */
  int lqd_mode;    /* 0: the reference's; 1: per-contact volumes and contact angles */
  float lqd_theta_max;
  double lqd_vol_min, lqd_vol_max;
  unsigned long long lqd_seed;
} o_consts;

/* heydem.h:209-214 SEARCHCELL (pointers to per-level arrays) */
typedef struct { int* numCells; oi3* gridSize; double* Cellsize; } o_searchcell;

/* the fields of PPCONTACT_HISTORY / PWCONTACT_HISTORY the step path uses
 * (heydem.h:153-190) */
typedef struct {
  ov3* dispt;
  double *nDsp, *nDsp_mx, *plstRad, *plstDfm;
  int *stage, *lqdBrg;
} o_history;

/* ---- per-kernel restatements (index-parallel, OpenMP where safe) ---- */

/* kernel.cu:646-673 calcHashG (+ calcGridPos :617-632, calcGridHash :638-641) */
void orc_calc_hash(int* hash, int* index, const int* pLevel, o_searchcell cell,
                   const int* Ncell_Idx, const ov3* pos, int n, const o_consts* k);
/* ParticleSystem.cu:61-69 thrust::sort_by_key (stable radix order) */
void orc_sort_by_key(int* hash, int* index, int n);
/* ParticleSystem.cu:83-103 + kernel.cu:682-724 (memset -1, then boundaries) */
void orc_find_cell_start(int* cellStart, int* cellEnd, const int* hash, int n, int numCells);
/* kernel.cu:729-855 NeighborFindG.  Returns the number of particles whose list
 * would have run past level_nNebors (the reference has no check; the oracle
 * stops appending for those and reports them). */
int orc_neighbor_find(const ov3* pos, const int* sortedIndex, const int* cellStart,
                      const int* cellEnd, const int* pLevel, o_searchcell cell,
                      const int* Ncell_Idx, const double* Level_size,
                      const int* level_nPars, const int* level_nNebors, int nLevels,
                      int* Nebor1, const int* Nebor_Idx, int* Num_Nebor, int n,
                      const double* rad, const o_consts* k);
/* kernel.cu:1034-1073 CirWallListG (wall list dense [NP][3]) */
void orc_wall_list(const ov3* pos, const double* rad, const o_cylinder* cir, int* wlist,
                   int* nwall, int n, const o_consts* k);
/* ParticleSystem.cu:358-375 PPCntHstryCopy / :336-354 WallCntHstryCopy */
void orc_history_rotate(o_history old_h, o_history cur_h, long count);
/* kernel.cu:869-911 HstryCopyG */
void orc_history_carry_pp(const int* Nebor1, const int* Nebor1_Old, const int* pLevel,
                          const int* level_nNebors, const int* level_nPars,
                          const int* Nebor_Idx, o_history old_h, o_history cur_h,
                          const int* Num_Nebor, const int* Num_Nebor_Old, int n);
/* kernel.cu:918-950 HstryCopyPWG (wall lists dense [NP][3]) */
void orc_history_carry_pw(const int* wlist, const int* wlist_old, o_history old_h,
                          o_history cur_h, const int* nwall, const int* nwall_old, int n,
                          int NP);
/* Allocation.cpp:308-317 VarInit */
void orc_var_init(ov3* force, ov3* mom, double* rmom, int* lqdCnt, int* lqdCnt_Old, int NP);
/* kernel.cu:413-552 PPForceCalcG with ContactForceD (:89-228) and fCap (:65-81) */
void orc_pp_force(const ov3* pos, const ov3* vel, const ov3* angvel, const double* rad,
                  const int* Nebor1, const int* pLevel, const int* level_nNebors,
                  const int* level_nPars, const int* Nebor_Idx, o_history h,
                  const int* Num_Nebor, int* lqdCnt, const int* lqdCnt_Old, ov3* force,
                  ov3* mom, double* rmom, int n, int NP, int ForceCap, int stage,
                  const o_consts* k);
/* kernel.cu:958-1023 CirPWInterG with MultiPWForceD (:370-403), PWcontactD (:236-359) */
void orc_wall_force(const ov3* pos, const ov3* vel, const ov3* angvel, ov3* force, ov3* mom,
                    double* rmom, const double* rad, o_cylinder* cir, o_history h,
                    const int* nwall, const int* wlist, int n, int NP, int stage,
                    const o_consts* k);
/* kernel.cu:563-606 UpdateSystemG; returns the number of particles that set the
 * rebuild flag */
int orc_update(const double* rad, ov3* pos, ov3* vel, ov3* angvel, const ov3* force,
               const ov3* mom, double* rmom, double* pMove, int n, const o_consts* k);

/* single-function probes for the contact laws (known-answer tests) */
double orc_fcap(double Splus, double ijVol, double effectR, const o_consts* k);
/* the per-contact liquid model (see dem_oracle.c): a particle's contact angle,
 * a pair's bridge volume, the regression with its contact-angle terms
 * (normalised, s = max(gapmn, S), v = 8 V) and the rupture distance */
float orc_theta(int id, unsigned long long seed, float theta_max);
double orc_pair_volume(const o_consts* k, int ida, int idb, double r_min);
double orc_willett(double s, double v, double theta);
double orc_rupture(double V, double theta);

/* ---- a whole simulation in the reference's layouts: main.cpp:433-568 ---- */
typedef struct orc_sim orc_sim;

/* sizes: NP particles (capacity == active here), nLevels size levels,
 * Sys_nCells total cells, nPPCnt neighbour slots */
orc_sim* orc_sim_new(int NP, int nLevels, int Sys_nCells, long nPPCnt);
void orc_sim_free(orc_sim* s);
/* named arrays, for filling inputs and reading results (NULL if unknown):
 * pos vel angvel force mom rmom rad pMove lqdCnt lqdCnt_Old pLevel Nebor_Idx
 * Level_size level_nNebors level_nPars Ncell_Idx numCells gridSize Cellsize
 * hash index cellStart cellEnd Nebor1 Nebor1_Old Num_Nebor Num_Nebor_Old wlist
 * wlist_old nwall nwall_old pp.* pp_old.* pw.* pw_old.* (dispt nDsp nDsp_mx
 * plstRad plstDfm stage lqdBrg), consts, cylinder */
void* orc_sim_ptr(orc_sim* s, const char* name);
/* scalar controls */
void orc_sim_set_mode(orc_sim* s, int ForceCap, int stage);
/* one time step of main.cpp:466-564 (no feed).  Returns 1 if it rebuilt the
 * neighbour lists this step, 0 otherwise, -1 on neighbour-slot overflow. */
int orc_sim_step(orc_sim* s);
/* counters: iter, rebuilds, last rebuild flag count */
long orc_sim_counter(orc_sim* s, const char* name);
/* set iter / flag (the last integration's rebuild count) / need_build, so a
 * simulation can be resumed from another implementation's state */
void orc_sim_set_counter(orc_sim* s, const char* name, long v);
/* request a rebuild at the start of the next step (feed / restart path) */
void orc_sim_request_rebuild(orc_sim* s);

/* kernel table so the same driver can run the reference's own kernels
 * (oracle/_ref) for the pin test */
typedef struct {
  void (*calc_hash)(int*, int*, const int*, o_searchcell, const int*, const ov3*, int,
                    const o_consts*);
  void (*find_cell_start)(int*, int*, const int*, int, int);
  int (*neighbor_find)(const ov3*, const int*, const int*, const int*, const int*,
                       o_searchcell, const int*, const double*, const int*, const int*, int,
                       int*, const int*, int*, int, const double*, const o_consts*);
  void (*wall_list)(const ov3*, const double*, const o_cylinder*, int*, int*, int,
                    const o_consts*);
  void (*carry_pp)(const int*, const int*, const int*, const int*, const int*, const int*,
                   o_history, o_history, const int*, const int*, int);
  void (*carry_pw)(const int*, const int*, o_history, o_history, const int*, const int*,
                   int, int);
  void (*pp_force)(const ov3*, const ov3*, const ov3*, const double*, const int*,
                   const int*, const int*, const int*, const int*, o_history, const int*,
                   int*, const int*, ov3*, ov3*, double*, int, int, int, int,
                   const o_consts*);
  void (*wall_force)(const ov3*, const ov3*, const ov3*, ov3*, ov3*, double*,
                     const double*, o_cylinder*, o_history, const int*, const int*, int,
                     int, int, const o_consts*);
  int (*update)(const double*, ov3*, ov3*, ov3*, const ov3*, const ov3*, double*, double*,
                int, const o_consts*);
} orc_kernels;
void orc_sim_set_kernels(orc_sim* s, const orc_kernels* table);
const orc_kernels* orc_default_kernels(void);

#ifdef __cplusplus
}
#endif
#endif
