/*
 * heydem_gb300.h -- public C ABI of libdem_gb300 (GB300 / sm_103a DEM packing engine).
 *
 * Two layers, both plain C (extern "C", raw pointers and sizes, no torch types):
 *
 *  1. The reference heyDEM interface, symbol for symbol.  Every function the
 *     reference declares in heydem.h:366-613 (set-up, constant upload, the
 *     per-step GPU wrappers, host I/O) is exported here with the identical
 *     signature and argument meaning, so the reference's driver (main.cpp) links
 *     against libdem_gb300 unchanged.  Each declaration cites the reference
 *     line it replaces.  These entry points keep the reference's data layouts
 *     (double3 AoS particle arrays, level/slot-major neighbour slots,
 *     slot-major contact history, pitched wall list) and run this library's
 *     own sm_103a kernels on them, on the legacy default stream, in FP64 with
 *     the reference's formulas.  Like the reference they return void; a CUDA
 *     failure prints the error and exits (heydem.h:25-35 behaviour), and
 *     dem_last_error() reports the most recent failure for callers that do not
 *     want to exit.
 *
 *  2. The native dem_* interface: a context that owns cell-sorted SoA device
 *     state, runs whole time steps as one CUDA graph (rebuild decided on the
 *     device), supports an FP32-force / FP64-state mode, returns status codes
 *     and imports/exports the reference's double3 host arrays at feed and output
 *     points.
 *
 * Units: everything on the device is in the reference's reduced units
 * (UnitReduce.cpp:14-20: length = REALSIZE, the largest diameter; mass =
 * rho*pi*D^3/6; force = m*g; time = sqrt(D/g)).
 */
#ifndef HEYDEM_GB300_H
#define HEYDEM_GB300_H

#include <stddef.h>
#include <stdio.h>
#include <vector_types.h> /* double2, double3, int3: layout of the reference's structs */

/* The reference's heydem.h defines `gravity` as a macro (heydem.h:16); a
 * translation unit that includes it first still sees this header's field of
 * that name as a field.  The macro is back in force after this header. */
#pragma push_macro("gravity")
#undef gravity

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Reference data model (heydem.h:39-320), layout-identical                   */
/* ------------------------------------------------------------------------ */
#ifndef HEYI_COMMON_H /* the reference's own heydem.h already declared these */
#define DEM_NUM_MAT 2 /* heydem.h:14 NUM_MAT */

typedef struct CylinderBC { double2 cir; double R; double Tw; double Bw; double topv, btmv; } CylinderBC; /* heydem.h:39-46 */
typedef struct FeedZone { double Lmax; double Lmin; } FeedZone;                                      /* heydem.h:63-67 */
typedef struct UNIT { double rlunit, rmunit, rfunit; double reunit, rsunit, rtunit, rvunit; } UNIT;   /* heydem.h:81-85 */
typedef struct MatType { double density; double emod, ymod, pois; double dmpn; double sfrc, rfrc; double yldp; } MatType; /* heydem.h:90-97 */
typedef struct LIQUID { double stension; double vol; double gapmn; double layer; double brknmx; } LIQUID; /* heydem.h:104-111 */
typedef struct SIMULATION {                                                                          /* heydem.h:118-135 */
  double dt, dtFactor, cutGap, ctime, simTime, fdtime, outtime, dumptime, outinterval, fdinterval;
  int iter; int Outs;
} SIMULATION;
typedef struct LOADMODE { int stage; double tPacking; int nOutPacking; } LOADMODE;                   /* heydem.h:142-148 */
typedef struct PPCONTACT_HISTORY {                                                                   /* heydem.h:153-173 */
  double3 *dispt; double3 *ShrForB; double3 *ShrMomB; double3 *nOld;
  double *nDsp; double *nDsp_mx; double *plstRad; double *plstDfm; double *bndRad;
  double *NorForB; double *NorMomB; double *TenStrn; double *ShrStrn;
  int *stage; int *lqdBrg; int *Exbond;
} PPCONTACT_HISTORY;
typedef struct PWCONTACT_HISTORY {                                                                   /* heydem.h:179-190 */
  double3 *dispt; double *nDsp; double *nDsp_mx; double *plstRad; double *plstDfm; int *stage; int *lqdBrg;
} PWCONTACT_HISTORY;
typedef struct PARAMETER { double3 Origin; double3 EndPoint; double SearchGap; double dt; int NP; } PARAMETER; /* heydem.h:196-204 */
typedef struct SEARCHCELL { int *numCells; int3 *gridSize; double *Cellsize; } SEARCHCELL;        /* heydem.h:209-214 */
typedef struct calParaPP { double emod, pois, sfrc, ystress, ydsp_t, yforce_t, ystiff_t; } calParaPP; /* heydem.h:220-229 */
typedef struct calParaPW { double emod, pois, sfrc, ystress, ydsp_t, yforce_t, ystiff_t; } calParaPW; /* heydem.h:233-242 */
#endif /* HEYI_COMMON_H */

/* ------------------------------------------------------------------------ */
/* Layer 1: the reference's extern "C" API (heydem.h:366-613)                 */
/* ------------------------------------------------------------------------ */

/* Process-global particle arrays the reference driver touches directly
 * (Allocation.cpp:5-18, declared in heydem.h:329-347).  C++ linkage, as in the
 * reference; defined by libdem_gb300 and filled by ParticleInfoAlloc /
 * SearchCellAlloc. */
#ifdef __cplusplus
}
extern double3 *hPos, *hVel, *hAngVel, *hForce;
extern double* hRad;
extern double3 *dPos, *dVel, *dAngVel, *dForce, *dMom;
extern double *dRMom, *dRad;
extern int *d_GridParticleHash, *d_GridParticleIndex, *d_CellStart, *d_CellEnd;
extern "C" {
#endif

/* set-up and allocation */
void ParticleInfoAlloc(int NP);                                                                    /* heydem.h:366 */
void PPCntHstry_Alloc(PPCONTACT_HISTORY* h_cntHstry_pp, PPCONTACT_HISTORY* d_cntHstry_pp,
                      PPCONTACT_HISTORY* d_cntHstry_ppOld, int nPPCnt);                            /* heydem.h:369 (C++ refs = pointers) */
void WallCntHstry_Alloc(PWCONTACT_HISTORY* h_cntHstry_Stlpw, PWCONTACT_HISTORY* d_cntHstry_Stlpw,
                        PWCONTACT_HISTORY* d_cntHstry_Stlpw_Old, int nWallCnt);                    /* heydem.h:372 */
void NeborListAlloc(int** h_Num_Nebor, int** h_1DNebor, double** d_pMoveforReBld, int** d_Num_Nebor,
                    int** d_Num_Nebor_Old, int** d_Nebor1, int** d_Nebor1_Old, int** h_Num_stlWall,
                    int** h_StlWList_1D, int** d_Num_StlWall, int** d_Num_StlWall_Old,
                    int** d_StlW_List, int** d_StlW_List_Old, size_t* pitch_Sw1, size_t* pitch_Sw2,
                    int NP, int nPPCnt, int StlMaxWallPerBall);                                    /* heydem.h:375 */
void VarInit(double3** dForce, double3** dMom, double** dRMom, int** d_lqdCnt, int** d_lqdCnt_Old,
             int NP);                                                                              /* heydem.h:386 */
void FeedZoneAlloc(FeedZone** Feedcube);                                                           /* heydem.h:393 */
void ParamAlloc(SIMULATION** h_dem, UNIT** Rdu, int** h_lqdCnt, int** d_lqdCnt, int** d_lqdCnt_Old,
                MatType** h_Mat, LIQUID** h_lqd, PARAMETER** h_Params, SEARCHCELL* h_cell,
                SEARCHCELL* d_cell, int nLevels, int NP);                                          /* heydem.h:396 */
void SearchCellAlloc(int NP, int numCells);                                                        /* heydem.h:402 */

/* host input / output (keyword file heyi.in, diameters, dump header, Tecplot) */
void FindRec(FILE* inFile, char* strDest);                                                         /* heydem.h:407 */
void ReadData(double* h_Level_size, int* h_pLevel, int* h_level_nNebors, int* h_level_nPars,
              int* h_Nebor_Idx, CylinderBC** h_Cir, CylinderBC** d_Cir, FeedZone* Feedcube,
              MatType* h_Mat, LIQUID* h_lqd, PARAMETER* h_Params, double* InitParSize,
              int* ForceCap, SIMULATION* h_dem, LOADMODE* h_load, double* hRad, SEARCHCELL h_cell,
              int NP, int nLevels, char* genfile, int RESTART);                                   /* heydem.h:410 */
void LoadPara(char* DumpName, int* NP, int* nBatch, int* TotalParticle);                           /* heydem.h:418 */
void WrtTec(double3* hPos, double3* hVel, double3* hForce, double3* hAngVel, SIMULATION* h_dem,
            double* hRad, UNIT* Rdu, int TotalParticle, int NP);                                   /* heydem.h:422 */
void DiaInput(char* diaFile, double* hRad, int NP);                                                /* heydem.h:427 */
void UnitReduce(UNIT* Rdu, CylinderBC* h_Cir, FeedZone* Feedcube, LOADMODE* h_load, double* hRad,
                MatType* h_Mat, LIQUID* h_lqd, double InitParSize, SIMULATION* h_dem,
                PARAMETER* h_Params, SEARCHCELL h_cell, double* h_Level_size, int nLevels, int NP,
                int RESTART, char* genfile);                                                       /* heydem.h:432 */
int ParticleFeed(FeedZone* Feedcube, CylinderBC* h_Cir, double InitParSize, double3* hPos,
                 double* hRad, int numParticle, int NP);                                           /* heydem.h:440 */
/* WrtTec's output (WriteTec.cpp:9-38) -- the same quantities X Y Z R VX VY VZ
 * |w| |F| and zones -- as full-precision binary columns in particle_info.bin
 * (no counterpart in the reference: at 10^7 particles the ASCII zone is
 * ~1.5 GB of formatted text).  Layout: "DEMCOL01", int32 column count,
 * 8-byte column names; per call "ZONE\0\0\0\0", float64 time [s], int64 count,
 * then each column as count float64 values. */
void WrtBin(double3* hPos, double3* hVel, double3* hForce, double3* hAngVel, SIMULATION* h_dem,
            double* hRad, UNIT* Rdu, int TotalParticle, int NP);

/* constant upload (kernel.cu:22-50) */
void setMaterial(MatType* h_Mat);                                                                  /* heydem.h:453 */
void setLiquid(LIQUID* h_lqd);                                                                     /* heydem.h:454 */
void setParameters(PARAMETER* h_Params);                                                           /* heydem.h:455 */
void setCalpara(calParaPP* h_cal, calParaPW* h_pWcal);                                             /* heydem.h:456 */
void IndexOffset(int* d_Num, int* d_nei, int Nn);                                                  /* heydem.h:457 */

/* per-step GPU wrappers (ParticleSystem.cu:141-375) */
void BldNeborList(int* d_GridParticleHash, int* d_GridParticleIndex, int* d_CellStart,
                  int* d_CellEnd, int* d_pLevel, SEARCHCELL d_cell, int* d_Ncell_Idx,
                  double* d_Level_size, int* d_level_nPars, int* d_level_nNebors, int nLevels,
                  double3* dPos, int Sys_nCells, int* d_Nebor1, int* d_Nebor_Idx, int* d_Num_Nebor,
                  int TotalParticle, double* dRad);                                                /* heydem.h:547 */
void BldCirWall(double3* dPos, double* dRad, CylinderBC* d_Cir, int* d_StlW_List, size_t pitch_Sw1,
                int* d_Num_StlWall, int TotalParticle);                                            /* heydem.h:556 */
void HstryCopy(int* d_Nebor1, int* d_OldNebor1, int* d_pLevel, int* d_level_nNebors,
               int* d_level_nPars, int* d_Nebor_Idx, PPCONTACT_HISTORY d_cntHstry_ppOld,
               PPCONTACT_HISTORY d_cntHstry_pp, int* d_Num_Nebor, int* d_Num_Nebor_Old,
               int TotalParticle, int NP);                                                         /* heydem.h:561 */
void HstryCopyPW(int* d_StlW_List, int* d_StlW_List_Old, size_t pitch_w1, size_t pitch_w2,
                 PWCONTACT_HISTORY d_cntHstry_pw_Old, PWCONTACT_HISTORY d_cntHstry_pw,
                 int* d_Num_StlWall, int* d_Num_StlWall_Old, int TotalParticle, int NP);          /* heydem.h:569 */
void PpInterCalc(double3* dPos, double3* dVel, double3* dAngVel, double* dRad, int* d_Nebor1,
                 int* d_pLevel, int* d_level_nNebors, int* d_level_nPars, int* d_Nebor_Idx,
                 PPCONTACT_HISTORY d_cntHstry_pp, int* d_Num_Nebor, int* d_lqdCnt,
                 int* d_lqdCnt_Old, double3* dForce, double3* dMom, double* dRMom,
                 int TotalParticle, int NP, int ForceCap, int stage);                              /* heydem.h:577 */
void CirPWCalc(double3* dPos, double3* dVel, double3* dAngVel, double3* dForce, double3* dMom,
               double* dRMom, double* dRad, CylinderBC* d_Cir, PWCONTACT_HISTORY d_cntHstry_Stlpw,
               int* d_Num_StlWall, int* d_StlW_List, size_t pitch_Sw1, int TotalParticle, int NP,
               int stage);                                                                         /* heydem.h:590 */
void UpdateSystem(double* dRad, double3* dPos, double3* dVel, double3* dAngVel, double3* dForce,
                  double3* dMom, double* dRMom, int* d_ReNebld, double* d_pMoveforReBld,
                  int TotalParticle);                                                              /* heydem.h:600 */
void NeborToCPU(int* h_Num_Nebor, int* d_Num_Nebor, int* h_1DNebor, int* d_Nebor1, int* h_Num_stlWall,
                int* d_Num_StlWall, int* h_StlWList_1D, int* d_StlW_List,
                PPCONTACT_HISTORY h_cntHstry_pp, PPCONTACT_HISTORY d_cntHstry_pp,
                PWCONTACT_HISTORY h_cntHstry_Stlpw, PWCONTACT_HISTORY d_cntHstry_Stlpw, int NP,
                int nPPCnt, size_t pitch_Sw1, int StlMaxWallPerBall);                              /* heydem.h:605 */
void WallCntHstryCopy(PWCONTACT_HISTORY d_cntHstry_Stlpw_Old, PWCONTACT_HISTORY d_cntHstry_Stlpw,
                      int nWallCnt);                                                               /* heydem.h:612 */
void PPCntHstryCopy(PPCONTACT_HISTORY d_cntHstry_ppOld, PPCONTACT_HISTORY d_cntHstry_pp,
                    int nPPCnt);                                                                   /* heydem.h:613 */

/* Note on C++ reference parameters: heydem.h declares the *_Alloc, VarInit,
 * ParamAlloc and ReadData pointer arguments as C++ references (T*& / T&).  On
 * the Itanium C++ ABI a reference is passed exactly as a pointer, so the
 * pointer forms above are the same machine-level signature and main.cpp's
 * calls bind to them unchanged. */

/* ------------------------------------------------------------------------ */
/* Layer 2: native interface                                                 */
/* ------------------------------------------------------------------------ */

typedef int dem_status;
enum {
  DEM_OK = 0,
  DEM_ERR_ARG = -1,      /* bad argument / size */
  DEM_ERR_CUDA = -2,     /* a CUDA call failed (see dem_last_error) */
  DEM_ERR_OVERFLOW = -3, /* a neighbour list ran past its level's slot capacity */
  DEM_ERR_NONFINITE = -4,/* NaN/Inf in particle state */
  DEM_ERR_IO = -5,       /* file missing / keyword missing / parse error */
  DEM_ERR_STATE = -6,    /* call out of order */
  DEM_ERR_NOMEM = -7,    /* device allocation failed */
  DEM_ERR_CELL = -8      /* a particle left the cell grid */
};

#define DEM_MAX_LEVELS 16

/* What heyi.in holds (ReadData.cpp:75-187, main.cpp:63-84), in SI units. */
typedef struct dem_input {
  int np;                 /* NUMPARTICLE */
  int n_levels;           /* SIZELEVEL */
  int load_stage;         /* LOADMODE */
  double t_packing;       /* packing_TIME [s] */
  int force_cap;          /* FoceCapillary yes/no */
  double real_size;       /* REALSIZE [m]: the largest diameter, the length unit */
  double cut_gap;         /* CUTGAPFORNEIGHBORLIST (in units of REALSIZE*Rmax/Rmin) */
  double expand_size;     /* EXPANDSIZE (domain margin in units of Rmax) */
  double cyl_x, cyl_y, cyl_bw, cyl_r, cyl_h; /* CylinderBC x y Bw R H [m] */
  double feed_lmin, feed_lmax;               /* FeedZone [m] */
  double mat[2][7];       /* MATERIAL: density ymod pois sfrc rfrc dmpn yldp, particle then wall */
  double lqd[3];          /* LIQUID: stension vol gapmn */
  double dt_factor;       /* SIMULATION dtFactor */
  int n_out;              /* SIMULATION nOut */
  int level_input;        /* SIZELEVEL_INPUT yes/no */
  double level_dia[DEM_MAX_LEVELS]; /* SIZELEVEL_INPUT diameters [m] */
  double dt_override;     /* > 0: use this dt [s] instead of the dtFactor rule (ReadData.cpp:263) */
  double gravity;         /* 0: the reference's 9.8 (heydem.h:16) */
} dem_input;

/* Everything the step path needs, derived exactly as ReadData.cpp:243-375,
 * UnitReduce.cpp:14-104 and main.cpp:328-348 derive it (reduced units). */
typedef struct dem_setup {
  int np, n_levels, force_cap, load_stage;
  double init_par_size;   /* REALSIZE [m] */
  CylinderBC cyl;
  FeedZone feed;
  MatType mat[2];
  LIQUID lqd;
  PARAMETER prm;
  calParaPP cal;
  calParaPW pwcal;
  UNIT unit;
  SIMULATION sim;
  LOADMODE load;
  double level_size[DEM_MAX_LEVELS];
  int level_nnebors[DEM_MAX_LEVELS];
  int level_npars[DEM_MAX_LEVELS];
  double cell_size[DEM_MAX_LEVELS];
  int3 grid_size[DEM_MAX_LEVELS];
  int num_cells[DEM_MAX_LEVELS];
  int ncell_idx[DEM_MAX_LEVELS]; /* inclusive scan of num_cells (IndexOffset) */
  int sys_ncells;
  long long n_pp_slots;           /* nPPCnt = sum level_npars * level_nnebors */
  double rad_min, rad_max;        /* reduced */
} dem_setup;

/* heyi.in (+ <genfile>_dia.dat when present) -> dem_input + diameters [m].
 * dia must hold np doubles; pass NULL to query np/n_levels only. */
dem_status dem_read_input(const char* genfile, dem_input* in, double* dia);
/* dem_input + diameters [m] -> dem_setup + per-particle rad (reduced), level and
 * level rank (Nebor_Idx). */
dem_status dem_build_setup(const dem_input* in, const double* dia, dem_setup* out, double* rad,
                           int* plevel, int* nebor_idx);

/* precision of the native step */
enum { DEM_PREC_FP64 = 0, DEM_PREC_MIXED = 1 };
/* capillary closure */
enum { DEM_CAP_FORMULA = 0, DEM_CAP_MLP = 1 };
/* pair loop of the mixed step kernel: the warp's lanes share out its particles'
 * pairs (WARP), or one thread walks one particle's pairs (THREAD); AUTO (the
 * default) takes THREAD, the faster of the two on packed and loose beds alike
 * (114.6 vs 157.2 us on the packed 200k wet bed, 6.4 contacts per sphere;
 * 505 vs 634 us on a sequentially deposited 2M bed, 2.2 contacts per sphere).
 * WARP, the same formulas in phases over the warp's compacted pairs, stays
 * selectable and tested. */
enum { DEM_PAIRS_AUTO = 0, DEM_PAIRS_WARP = 1, DEM_PAIRS_THREAD = 2 };

typedef struct dem_options {
  int precision;          /* DEM_PREC_* */
  int capillary;          /* DEM_CAP_* */
  int block_size;         /* threads per block of the step kernel, a multiple of 32 up to 128
                             (0 = default: 32 for the WARP loop, 128 for THREAD and with the
                             learned closure) */
  int reorder;            /* 1: keep particles in cell order (default); 0: reference order */
  int use_graph;          /* 1: replay steps through a CUDA graph (default) */
  int graph_steps;        /* time steps per graph launch (0 = 16) */
  int pair_mode;          /* mixed step kernel: DEM_PAIRS_AUTO (default), _WARP or _THREAD */
} dem_options;

typedef struct dem_ctx dem_ctx;

typedef struct dem_stats {
  long long iter;         /* steps taken */
  long long rebuilds;     /* neighbour-list rebuilds */
  long long nb_entries;   /* neighbour-list entries at the last rebuild */
  long long contacts;     /* directed p-p contacts (gap < 0) in the last step */
  long long bridges;      /* directed wet non-contact bridges in the last step */
  long long wall_contacts;/* particle-wall contacts in the last step */
  int error_bits;         /* device error word (1: overflow, 2: non-finite, 4: cell range) */
  int pad;
  double ctime;           /* simulated time (reduced) */
  long long cap_mlp;      /* DEM_CAP_MLP: bridges evaluated by the network (cumulative) */
  long long cap_fallback; /* DEM_CAP_MLP: bridges outside its training box, plain formula (cumulative) */
} dem_stats;

void dem_default_options(dem_options* o);
dem_status dem_create(const dem_setup* s, const double* rad, const int* plevel,
                      const int* nebor_idx, const dem_options* opt, dem_ctx** out);
dem_status dem_destroy(dem_ctx* c);
/* Host state in the reference's double3 layout and particle order (reduced
 * units).  vel/angvel may be NULL (zero).  Marks the lists for rebuild.
 * Returns once the caller's arrays have been read.  Page-locked arrays
 * (cudaHostAlloc, cudaMallocHost, cudaHostRegister, a framework's pinned
 * buffers) are read by the import kernel itself over the host link, with no
 * staging copy; pageable arrays go through the copy engines, and the device
 * work behind those copies stays queued on the context's stream. */
dem_status dem_set_state(dem_ctx* c, const double3* pos, const double3* vel, const double3* angvel);
/* As dem_set_state, but with request_rebuild = 0 the current neighbour lists,
 * contact history and path-length accumulators are kept: for callers that
 * round-trip the state through host memory between steps (the lists stay
 * valid as long as no particle moved by more than the skin allowance). */
dem_status dem_set_state_ex(dem_ctx* c, const double3* pos, const double3* vel, const double3* angvel,
                            int request_rebuild);
/* Any pointer may be NULL.  force/mom are the last step's totals.  Returns
 * when every requested array is written.  When every requested array is
 * page-locked one kernel gathers them into caller order and writes them over
 * the host link directly; otherwise each goes through device staging and the
 * copy engines. */
dem_status dem_get_state(dem_ctx* c, double3* pos, double3* vel, double3* angvel, double3* force,
                         double3* mom);
/* One round trip for a caller that keeps the state in host memory: import
 * pos/vel/angvel (as dem_set_state_ex with request_rebuild = 0; vel/angvel may
 * be NULL: zero, and then not exported), advance nsteps, export
 * pos/vel/angvel/force back into the same arrays (force may be NULL).  The
 * three are queued back to back and the host waits once, at the end, so the
 * device does not idle while the host returns from the import and launches
 * the steps.  Page-locked arrays are read and written directly (as in
 * dem_set_state_ex / dem_get_state).  The caller's arrays must not be touched
 * until it returns. */
dem_status dem_advance(dem_ctx* c, double3* pos, double3* vel, double3* angvel, double3* force, int nsteps);
/* Advance nsteps time steps.  Device-resident; no host synchronisation inside
 * unless the context was created without graphs. */
dem_status dem_step(dem_ctx* c, int nsteps);
/* Time the force+integration kernel(s) of one step alone: reps launches on the
 * context's stream, each bracketed by CUDA events; before each, flush_bytes of
 * flush_buf (device memory, may be NULL) are overwritten so the launch starts
 * with a cold L2.  The launches advance the simulation like dem_step without
 * rebuilds.  *ms_avg receives the mean launch time in milliseconds. */
dem_status dem_profile_step(dem_ctx* c, int reps, void* flush_buf, size_t flush_bytes, double* ms_avg);
/* Evict the L2 cache for timing: on `stream` (a cudaStream_t), overwrite the
 * first half of the device buffer, then read the second half, so the cache ends
 * up holding clean lines of unrelated data (no write-backs charged to the next
 * kernel).  bytes should be at least twice the L2 size. */
dem_status dem_l2_flush(void* stream, void* buf, size_t bytes);
/* Wait for the context's stream and check the device error word. */
dem_status dem_sync(dem_ctx* c);
dem_status dem_get_stats(dem_ctx* c, dem_stats* st);
/* The context's CUDA stream (cudaStream_t) for callers that time or order work. */
void* dem_stream(dem_ctx* c);
/* 1 when the context's steps launch one another on the device (mixed
 * precision with graphs, after the first dem_step), 0 when they run as
 * host-launched graphs with a conditional rebuild node or host-driven. */
int dem_step_chained(dem_ctx* c);
/* ---- liquid-bridge model (no counterpart in the reference) ----
 * DEM_LIQUID_REFERENCE: the reference's (kernel.cu:429-434, :511-544): each
 * particle's liquid LIQUID.vol (2r)^3 split over max(12, its bridges), the
 * capillary regression at zero contact angle.
 * DEM_LIQUID_PER_CONTACT: each unordered pair's bridge volume is a fraction of
 * the smaller sphere's volume, uniform in [vol_min, vol_max] from a hash of the
 * two particle ids and the seed; each particle's contact angle is uniform in
 * [0, theta_max] (radians) from a hash of its id and the seed, a pair takes
 * the mean; the force is the same regression with its contact-angle terms
 * (Willett et al. 2000), rupture at (1 + theta/2) 0.99 V^0.33.  Formation,
 * bridge flags and LIQUID.stension / gapmn / layer are the reference's. */
#define DEM_LIQUID_REFERENCE 0
#define DEM_LIQUID_PER_CONTACT 1
typedef struct dem_liquid_model {
  int mode;
  int pad;
  double vol_min, vol_max;
  double theta_max;
  unsigned long long seed;
} dem_liquid_model;
/* Set the liquid model (before the first dem_step; both precisions).  It also
 * sets the learned closure's per-particle contact angles to the model's. */
dem_status dem_set_liquid_model(dem_ctx* c, const dem_liquid_model* m);
/* Name of the step kernel(s) dem_step launches for this context's precision,
 * closure and pair loop, e.g. "k_step_mixed<1,0>" (a static string). */
const char* dem_step_kernel(dem_ctx* c);
/* Where the time of one end-to-end step goes: `reps` times the host-facing
 * sequence dem_set_state_ex(pos, vel, angvel, no rebuild request) ->
 * dem_step(1) -> dem_get_state(pos, vel, angvel, force) on pinned or pageable
 * host arrays, with timing events at the calls' boundaries.  out[9], each the
 * mean in ms: [0] host wall time of the sequence; device spans [1] upload
 * copies (page-locked arrays: the import kernel that reads them), [2] import
 * and shadows (plus the host's return; ~0 for page-locked arrays), [3] from
 * the import to the end of the step (the host's launch of the step included),
 * [4] from the step to the export's start, [5] export gathers and copies
 * (page-locked arrays: the one export kernel);
 * host time inside [6] dem_set_state_ex, [7] dem_step, [8] dem_get_state.
 * The state goes round trip unchanged but for the steps taken. */
dem_status dem_e2e_parts(dem_ctx* c, double3* pos, double3* vel, double3* angvel, double3* force, int reps,
                         double* out);
/* Current neighbour lists in the reference's terms: for every particle i (in
 * the caller's order) its partners (caller's ids) in the reference's list order.
 * counts[np]; partners[np*max_per] (row i = partners of i).  Returns
 * DEM_ERR_ARG if max_per is too small. */
dem_status dem_get_neighbors(dem_ctx* c, int* counts, int* partners, int max_per);
/* Contact history of the pair (i, partners[i][k]) in reference terms,
 * rec[np*max_per][8] = dispt.x dispt.y dispt.z nDsp nDsp_mx plstRad plstDfm
 * stage, plus bridge flags brg[np*max_per]. */
dem_status dem_get_history(dem_ctx* c, double* rec, int* brg, int max_per);
/* The rest of the per-particle state, in the caller's order: path length since
 * the last rebuild pmove[np], last step's bridge count lqd[np], wall list
 * nwall[np] / wlist[np][3] (0 top, 1 bottom, 2 lateral) with its records
 * wrec[np][3][8] (as dem_get_history), and the pending rebuild flag (the
 * count of particles past the move limit, or 1 for a rebuild requested
 * otherwise; 0: the next step keeps the lists).  Any pointer may be NULL. */
dem_status dem_get_aux(dem_ctx* c, double* pmove, int* lqd, int* nwall, int* wlist, double* wrec, int* flag);
/* Batched systems (no counterpart in the reference): the context's particles
 * belong to n_sys independent packings laid out side by side in its domain
 * (no two systems within a neighbour search distance of each other), stepped
 * together by the same launches.  system_of_particle[np] (caller order) gives
 * each particle's system, cyl[n_sys] (reduced units) each system's container
 * and wet[n_sys] (NULL: the set-up's force_cap for all) whether its bridges
 * act.  Mixed precision only; call once, before stepping the systems. */
dem_status dem_set_systems(dem_ctx* c, int n_sys, const int* system_of_particle, const CylinderBC* cyl,
                           const int* wet);
/* Write / read the full engine state (binary, with the reference's
 * "SYSTEM Info" text header so LoadPara can parse it). */
/* One step with a forced neighbour rebuild, launched from the host with a CUDA
 * event after each kernel: out[k] = {kernel (or group), device ms} in launch
 * order, *n_out entries (at most max_out).  The step counts as a step. */
typedef struct dem_kernel_time { char name[48]; double ms; } dem_kernel_time;
dem_status dem_profile_kernels(dem_ctx* c, dem_kernel_time* out, int max_out, int* n_out);
dem_status dem_save(dem_ctx* c, const char* path, int nBatch);
dem_status dem_load(dem_ctx* c, const char* path);

/* Seed of ParticleFeed's generator (the reference seeds from the clock,
 * ParticleFeed.cpp:17; here feeds are reproducible). */
void dem_set_feed_seed(unsigned long long seed);
/* ParticleFeed (ParticleFeed.cpp:8-72) on the device arrays, replacing the
 * sequence main.cpp:442-448 (positions down, ParticleFeed, positions up):
 * dPos / dRad are device arrays of capacity NP (dRad holds every particle's
 * radius, as hRad does); up to 60000 new particles numParticle.. are placed in
 * the feed band with the reference's draws and clearance (r_i + r_j + 0.002),
 * in parallel rounds, each given up after 500 tries; the batch keeps the
 * particles below the first one that failed.  Counter-based generator: the
 * same seed gives the same positions.  Allocates its scratch with cudaMalloc
 * and synchronises the device.  Returns the new particle count, or -1
 * (dem_last_error). */
int ParticleFeedDevice(FeedZone* Feedcube, CylinderBC* h_Cir, double InitParSize, double3* dPos,
                       double* dRad, int numParticle, int NP, unsigned long long seed);
/* The arithmetic of the reference-compatible PpInterCalc, CirPWCalc and
 * UpdateSystem.  DEM_PREC_FP64 (the default): the reference's FP64 formulas,
 * forces equal to the CPU oracle's to 1e-12.  DEM_PREC_MIXED: the fused step's
 * FP32 contact and bridge laws on the same layouts (Kahan sums; positions,
 * velocities, springs and peak overlaps stay FP64; the integrator adds FP32
 * increments to them), the tolerances of dem_options.precision = DEM_PREC_MIXED.
 * The environment variable DEM_COMPAT_PRECISION=mixed selects the mixed mode
 * for a driver that is not changed (the reference's main.cpp); this call
 * overrides it.  Lists (BldNeborList) are the same in both modes.
 * Returns DEM_ERR_ARG for another value. */
dem_status dem_compat_set_precision(int precision);
/* the mode the next reference-compatible call will use (DEM_PREC_*) */
int dem_compat_precision(void);
/* Reads and clears the error word of the reference-compatible entry points:
 * bit 1 = a neighbour list stopped at its level's slot capacity (the
 * reference would write past it, kernel.cu:833-836), bit 4 = a particle hashed
 * outside the cell grid. */
int dem_compat_errors(void);
/* BldNeborList (above) without any device allocation.  No counterpart in the
 * reference: its BldNeborList sorts with thrust, which allocates temporary
 * storage on every call, and this library's BldNeborList keeps a scratch cache
 * that it frees and re-allocates when the particle count grows.
 *
 * Same arguments and outputs as BldNeborList, plus d_err: one device int the
 * caller owns, which must be zero before the first call; the kernels OR bit 1
 * (a neighbour list stopped at its level's slot capacity) and bit 4 (a
 * particle hashed outside the cell grid) into it and never clear it.  The
 * cell sort's scratch is a fixed 16 MiB array of device memory inside the
 * library: 4 * (2 * TotalParticle + ceil(Sys_nCells / 2048) + 64) bytes must
 * fit, i.e. up to about 2,000,000 particles; larger sizes return DEM_ERR_ARG
 * with a message and launch nothing.  Every call looks the array's address
 * up in the current context (cudaGetSymbolAddress), so the call stays valid
 * after cudaDeviceReset.  With CUDA's lazy module loading (the default), the
 * array is committed when the library's device code first loads on a device,
 * which can be this call's first use: a caller that reserves the rest of the
 * card's memory up front should make one call (or run with
 * CUDA_MODULE_LOADING=EAGER) before reserving, and make that first call
 * before any stream capture.  Calls share that one array: two calls whose
 * kernels run at the same time on one device race.
 * Returns DEM_OK or a negative dem_status (see dem_last_error). */
int BldNeborListNoAlloc(int* d_GridParticleHash, int* d_GridParticleIndex, int* d_CellStart,
                        int* d_CellEnd, int* d_pLevel, SEARCHCELL d_cell, int* d_Ncell_Idx,
                        double* d_Level_size, int* d_level_nPars, int* d_level_nNebors, int nLevels,
                        double3* dPos, int Sys_nCells, int* d_Nebor1, int* d_Nebor_Idx,
                        int* d_Num_Nebor, int TotalParticle, double* dRad, int* d_err);
/* Seeded sequential deposition into a cylinder (test / benchmark inputs):
 * particles in the given order are dropped at the lowest of `tries` random
 * (x, y) candidates inside radius R - r of the axis (cx, cy) onto the floor z0
 * or the highest sphere below them, with a clearance `gap` between surfaces.
 * dia[n] and pos_out[n] in the same (any) length unit. */
dem_status dem_pack_deposit(int n, const double* dia, double cx, double cy, double R, double z0,
                            double gap, int tries, unsigned long long seed, double3* pos_out);
/* Packing fraction and mean coordination number of a bed (host, any units):
 * probe cylinder coaxial with the container, radius R - 3 d_max, from
 * Bw + 3 d_max to 3 d_max below the free surface (98th percentile of sphere
 * tops); spheres clipped exactly by the probe; Z = mean number of overlapping
 * p-p contacts of the spheres centred in the probe. */
dem_status dem_packing_metrics(int n, const double3* pos, const double* rad, const CylinderBC* cyl, double* phi,
                               double* z_mean, int* n_probe);
/* ---- memory plan (no counterpart in the reference) ----
 * Device bytes dem_create allocates for a set-up and options. */
typedef struct dem_memory {
  long long per_particle;  /* bytes per particle (state, copies, wall lists and records, sort) */
  long long per_slot;      /* bytes per neighbour slot (list, record, bridge flag, and their copies) */
  long long per_cell;      /* bytes per cell (ranges, scan tiles) */
  long long slots;         /* neighbour slots of the set-up */
  long long total;         /* all of it, plus small fixed tables */
} dem_memory;
dem_status dem_memory_estimate(const dem_setup* s, const dem_options* o, dem_memory* out);
/* Scale every level's neighbour slots by one factor f <= 1 (each level keeps
 * at least min_slots) so that dem_create's allocation fits budget_bytes;
 * updates s->level_nnebors and s->n_pp_slots and returns f.  The reference's
 * slot formula (ReadData.cpp:302) reserves ~100 slots per particle where a
 * packed bed uses a few; a level that outgrows its slots is reported by
 * dem_sync as DEM_ERR_OVERFLOW, never written past.  DEM_ERR_NOMEM if even
 * min_slots does not fit. */
dem_status dem_fit_memory(dem_setup* s, const dem_options* o, double budget_bytes, int min_slots, double* factor);

/* ---- cell size and the autotuner (no counterpart in the reference) ----
 * Multiply every level's cell size by factor in [1, 16] and rederive the
 * grids (larger cells keep the 27-cell neighbour search complete). */
dem_status dem_scale_cells(dem_setup* s, double factor);
typedef struct dem_tune_space {
  int n_skin, n_cell, n_block, pad;
  double skin_scale[8];   /* multiples of the input's CUTGAPFORNEIGHBORLIST */
  double cell_scale[8];   /* factors for dem_scale_cells */
  int block_size[4];      /* threads per block of the step kernel (multiples of 32, <= 128) */
  int warmup_steps;       /* untimed steps of each trial (the first builds the lists) */
  int trial_steps;        /* timed steps of each trial */
} dem_tune_space;
typedef struct dem_tune_result {
  double skin_scale, cell_scale;
  int block_size, n_tried;
  double best_rate;       /* particle-steps/s of the chosen candidate */
  double rate[64];        /* every candidate, skin-major then cell then block */
} dem_tune_result;
/* Time every candidate of `space` on the given bed (positions / velocities in
 * the set-up's reduced units; batched systems as dem_set_systems, n_sys = 0
 * for one system) and return the fastest one's set-up and options. */
dem_status dem_autotune(const dem_input* in, const double* dia, const double3* pos, const double3* vel,
                        const dem_options* base, const dem_tune_space* space, int n_sys,
                        const int* system_of_particle, const CylinderBC* cyl, const int* wet,
                        dem_setup* best_setup, dem_options* best_opt, dem_tune_result* rep);

/* ---- learned capillary closure (no counterpart in the reference) ----
 * A 4 -> 64 -> 64 -> 2 SiLU network standing in for the reference's capillary
 * routine fCap (kernel.cu:65-81) and rupture distance (kernel.cu:518).
 * Raw features per bridge, in the reduced length unit of the kernels:
 *   [0] S+ = max(gapmn, gap)  [1] V = 8 (Vi + Vj)  [2] contact angle [rad]
 *   [3] radius ratio r_min / r_max
 * raw targets: [0] F / (2 pi R_eff gamma)  [1] rupture distance 0.99 (V/8)^0.33.
 * Parameter vector (FP32, 4610): W1[64][4] b1[64] W2[64][64] b2[64] W3[2][64] b3[2];
 * standardisation vector (20): x_mean[4] x_std[4] y_mean[2] y_std[2], and the
 * training box of the raw features hull_lo[4] hull_hi[4]. */
typedef struct dem_capnet dem_capnet;
typedef struct dem_capnet_fit_opts {
  int epochs;             /* passes over the training split */
  int batch;              /* samples per Adam step */
  float lr;               /* Adam learning rate (beta 0.9 / 0.999, eps 1e-8) */
  float val_frac;         /* held-out fraction (seeded split) */
  unsigned long long seed;
} dem_capnet_fit_opts;
typedef struct dem_capnet_report {
  int epochs, n_train, n_val, pad;
  float train_mse[64];    /* standardised MSE per epoch (sampled batches), first 64 epochs */
  float val_mse;          /* standardised MSE of the FP32 network on the held-out split */
  float val_force_rel_mean, val_force_rel_max; /* BF16 tensor-core network vs the formula's force */
  float val_rupture_rel_max;
  double seconds;
} dem_capnet_report;

dem_status dem_capnet_create(unsigned long long seed, dem_capnet** out);
void dem_capnet_destroy(dem_capnet* net);
/* parameters (4610) and standardisation (20), host arrays; either may be NULL */
dem_status dem_capnet_get(const dem_capnet* net, float* params, float* norm);
dem_status dem_capnet_set(dem_capnet* net, const float* params, const float* norm);
/* Training samples from a wet context's current state: every bridged pair,
 * features x_dev[n][4] and the formula's targets y_dev[n][2] (FP64 formula,
 * stored FP32), device arrays, in particle / slot order.  *count = samples
 * written (at most capacity). */
dem_status dem_capnet_samples(dem_ctx* c, float* x_dev, float* y_dev, long long capacity, long long* count);
/* Adam on the network's own training kernels: seeded split, standardisation
 * and training box from the training split, then validation. */
dem_status dem_capnet_fit(dem_capnet* net, const float* x_dev, const float* y_dev, long long n,
                          const dem_capnet_fit_opts* opt, dem_capnet_report* rep);
/* Gradient of the loss (mean over the n samples of the squared error of the
 * standardised outputs) with respect to the 4610 parameters, and the loss. */
dem_status dem_capnet_grad(dem_capnet* net, const float* x_dev, const float* y_dev, int n, float* grad,
                           float* loss);
/* Raw features -> raw outputs: tensor_cores = 1 runs the BF16 warp tiles the
 * step kernel uses (mma.sync, 16 rows per warp), 2 the same network on the
 * 5th-generation tensor cores (tcgen05.mma into tensor memory, 128 rows per
 * CTA), 0 the FP32 network. */
dem_status dem_capnet_infer(dem_capnet* net, const float* x_dev, long long n, int tensor_cores, float* y_dev);
/* The plain closure the network stands in for, on the same raw features:
 * bit 0 of fp64 set: FP64 as the reference evaluates it (FP64 pow/log/exp),
 * clear: the step kernel's FP32 form; bit 1 set: the per-contact liquid
 * model's regression with the contact angle of feature 2 (the reference's is
 * the zero-angle case). */
dem_status dem_capnet_formula(const float* x_dev, long long n, int fp64, float* y_dev);
/* Install a trained network in a context created with DEM_PREC_MIXED and
 * DEM_CAP_MLP; bridges outside its training box keep the plain formula. */
dem_status dem_set_capnet(dem_ctx* c, dem_capnet* net);
/* Contact angles: uniform in [0, theta_max] per particle, hashed from the
 * particle id with `seed` (default 30 degrees, seed 0). */
dem_status dem_set_contact_angles(dem_ctx* c, float theta_max, unsigned long long seed);

/* Struct sizes and offsets of this header, for binding checks. */
int dem_abi_layout(long long* out, int cap);

/* Most recent error message (thread-local), never NULL. */
const char* dem_last_error(void);
/* Library build string. */
const char* dem_version(void);

#ifdef __cplusplus
}
#endif
#pragma pop_macro("gravity")
#endif /* HEYDEM_GB300_H */
