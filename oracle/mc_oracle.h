/*
 * mc_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is a plain C++17 FP64 restatement of
 * montecarlocpp's deviational phonon Monte Carlo field solve
 * (montecarlo/problem.cpp:370-445 and everything it calls). Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
 * only as the checker or the timed CPU baseline. The product library never
 * links, loads or calls it.
 *
 * Parity status: UNPINNED against the original binary. The reference needs
 * Eigen 3 and Boost (Random, Fusion, MPL, Optional), neither of which exists
 * on this machine, and the reference ships no tests, golden vectors or
 * fixtures. The oracle is pinned instead by known answers that follow from
 * the reference's own formulas (bulk conductivity Material::cond(),
 * montecarlo/material.cpp:233; tally partition of unity; RNG known-answer
 * vectors) and its trajectories are the replay target of the GPU path.
 */
#ifndef MC_ORACLE_H
#define MC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Face kinds, in the order of montecarlo/boundary.h:137-281. */
enum { ORC_SPEC = 0, ORC_DIFF = 1, ORC_ISOT = 2, ORC_PERI = 3, ORC_INTER = 4 };

/* One Parallelepiped<Bac, Lef, Bot, Fro, Rig, Top> subdomain
 * (montecarlo/subdomain.h:145-158): origin, matrix (row-major M[3*r+c];
 * columns are the edge vectors), divisions, volumetric gradient and the
 * kind and temperature of each of the six faces in Bac..Top order. */
typedef struct {
    double o[3];
    double M[9];
    long div[3];
    double gradT[3];
    int kind[6];
    double T[6];
} orc_pped;

/* Subdomain shapes (montecarlo/subdomain.h:128-640). */
enum {
    ORC_PARALLELEPIPED = 0,   /* 3 columns, 6 faces Bac Lef Bot Fro Rig Top      */
    ORC_TRIANGULAR_PRISM = 1, /* 3 columns, 5 faces Bac Lef Bot Dia Top          */
    ORC_TETRAHEDRON = 2,      /* 3 columns, 4 faces Bac Lef Bot Dia              */
    ORC_PRISM = 3,            /* N columns (axis, then the base vertices), N + 2
                                 faces Bot Top Sid0 .. Sid(N-1)                  */
    ORC_PYRAMID = 4           /* N columns (apex, then the base vertices), N + 1
                                 faces Bot Sid0 .. Sid(N-1)                      */
};
#define ORC_MAX_COLS 9
#define ORC_MAX_FACES 11

/* One subdomain of any shape: the constructor arguments (o, mat, div,
 * gradT, T) of Parallelepiped / TriangularPrism / Tetrahedron / Prism<N> /
 * Pyramid<N> and the kind of each face, in the order of the reference's
 * bdry<I>(). mat is column-major (column c at mat[3c .. 3c + 2]). Prism and
 * Pyramid take one division count, div[0] (< 0: no field, else one
 * column: montecarlo/subdomain.h:386-390,524-530). */
typedef struct {
    int shape;
    int ncols;
    double o[3];
    double mat[3 * ORC_MAX_COLS];
    long div[3];
    double gradT[3];
    int kind[ORC_MAX_FACES];
    double T[ORC_MAX_FACES];
} orc_sdom;

/* One makePair call (montecarlo/boundary.cpp:361-369 for Inter,
 * montecarlo/boundary.cpp:524-550 for Peri). rot is row-major. */
typedef struct {
    int kind;          /* ORC_PERI or ORC_INTER */
    int sdom1, face1;  /* first face: subdomain index, face index (bdry<I>()) */
    int sdom2, face2;
    double transl[3];  /* Peri only */
    double rot[9];     /* Peri only, identity when unused */
} orc_pair;

/* Uniform sources. */
enum {
    ORC_RNG_MT_THREADS = 0, /* reference scheme: nchunk mt19937 engines seeded
                               seed, seed+1, ... over static chunks of phonons
                               (montecarlo/main.cpp:29-39,155-160,
                               montecarlo/problem.cpp:383) */
    ORC_RNG_PHILOX = 1,     /* Philox4x32-10 keyed by seed, counter
                               (phonon id, event index, block, 0) */
    ORC_RNG_REPLAY = 2      /* per-phonon recorded 32-bit words */
};

enum { ORC_TEMP = 0, ORC_FLUX = 1, ORC_MULTI = 2, ORC_CUMTEMP = 3, ORC_CUMFLUX = 4 };

typedef struct {
    int problem;            /* ORC_TEMP / ORC_FLUX / ORC_MULTI / ORC_CUMTEMP / ORC_CUMFLUX */
    long nemit;
    long maxscat;
    long maxloop;           /* 0 -> 100 * maxscat (montecarlo/problem.cpp:339) */
    double dt;              /* step length used to count phonon-steps */
    double horizon;         /* time horizon in s; <= 0 means none */
    int rng;
    uint64_t seed;
    int nchunk;             /* ORC_RNG_MT_THREADS: number of engines */
    int nthreads;           /* OpenMP threads (0 = default) */
    /* replay input */
    const uint32_t* replay_words;
    const int64_t* replay_offsets;   /* nemit + 1 entries */
    /* recording of consumed words (may be NULL) */
    uint32_t* record_words;          /* capacity record_cap per phonon */
    int64_t* record_counts;          /* nemit entries */
    long record_cap;
    /* event log (may be NULL): log_cap records per phonon, 12 doubles each:
       loop index, subdomain before, face hit (-1 scatter, -2 horizon,
       -3 escape), subdomain after, flat cell index after, x, y, z, time,
       nscat, w, p */
    double* log;
    int64_t* log_counts;
    long log_cap;
    long log_phonons;                /* only phonons id < log_phonons log */
    /* CumTemp / CumFlux: number of scatter-count bins after the first
       (montecarlo/problem.cpp:553-648); rows = size + 1 or 3 (size + 1) */
    long cum_size;
} orc_problem;

typedef struct {
    long nemit;
    double power;
    long rows, cols;
    double phonon_steps;  /* sum over phonons of max(1, ceil(t_end / dt)) */
    long events;          /* loop iterations that completed an event */
    long scatters;
    long escapes;
    long horizon_stops;
    long maxscat_stops;
    long absorbed;
    long replay_exhausted; /* phonons whose replay stream ran out */
    double seconds;
    long threads;           /* OpenMP threads the solve ran on */
} orc_stats;

typedef struct orc_material orc_material;
typedef struct orc_domain orc_domain;

orc_material* orc_material_load(const char* disp, const char* relax, double T);
orc_material* orc_material_from_tables(const double* disp, long nw, long np,
                                       const double* relax, double T);
void orc_material_free(orc_material* m);
/* out: energySum, fluxSum, scatSum, cond */
void orc_material_sums(const orc_material* m, double out[4]);
/* Draw (w, p) from the scatter (which=2), flux (1) or energy (0) table
 * for a pair of 32-bit words. */
void orc_material_draw(const orc_material* m, int which, uint32_t x1,
                       uint32_t x2, long* w, long* p);
void orc_material_tables(const orc_material* m, double* vel, double* tau);

orc_domain* orc_domain_create(const orc_pped* s, int ns, const orc_pair* p,
                              int np);
/* The same for subdomains of any shape; NULL on an invalid description. */
orc_domain* orc_domain_create_shapes(const orc_sdom* s, int ns,
                                     const orc_pair* p, int np);
void orc_domain_free(orc_domain* d);
long orc_domain_cols(const orc_domain* d);
/* Subdomain::cellVol of every field column (cols entries). */
void orc_domain_cell_volumes(const orc_domain* d, double* out);
/* Volume of subdomain s (Subdomain::vol) and the emission weight of each
 * emitter (nemitters entries, volume emitters first per subdomain as
 * montecarlo/domain.cpp:88-102 registers them); returns the emitter count. */
double orc_domain_sdom_volume(const orc_domain* d, int s);
long orc_domain_emitters(const orc_domain* d, double* weights, int* sdom, int* face);
/* Emitter::drawPos of emitter e from the words of a Philox stream keyed
 * (seed, id) at event 0: n positions (3 doubles each) for ids 0 .. n-1.
 * The words consumed are those of emission after drawFluxProp. */
void orc_domain_draw_positions(const orc_domain* d, long e, uint64_t seed,
                               long n, double* out);
/* Subdomain::isInside (montecarlo/subdomain.cpp:108-116). */
int orc_domain_is_inside(const orc_domain* d, int s, const double* x);
/* Known-geometry builders restating montecarlo/domain.cpp:137-199. */
orc_domain* orc_domain_film(double Lx, double Ly, double Lz, long divy,
                            double dT);
orc_domain* orc_domain_bulk(double L, long divx, double dT);

/* Field::accumulate restated (montecarlo/field.cpp:92-220): accumulate
 * `amount` (rows entries) along bpos->epos in subdomain `sdom` into
 * data (rows x cols, column-major). */
void orc_accumulate(const orc_domain* d, int sdom, const double* bpos,
                    const double* epos, const double* amount, long rows,
                    double* data);

int orc_solve(const orc_material* m, const orc_domain* d,
              const orc_problem* prob, double* out, orc_stats* stats);

/* RNG known-answer helpers */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
uint32_t orc_mt19937_nth(uint32_t seed, long n);
/* drawIso / drawAniso (montecarlo/random.cpp:16-44) from two words */
void orc_draw_iso(uint32_t x1, uint32_t x2, double out[3]);
void orc_draw_aniso(uint32_t x1, uint32_t x2, int bidir, double out[3]);
/* rotation taking z-hat to n (row-major), as used by the oracle */
void orc_rot_z_to(const double n[3], double R[9]);

#ifdef __cplusplus
}
#endif

#endif
