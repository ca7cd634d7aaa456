// mc_layout.h -- plain-old-data layouts shared by the host library and the
// sm_103a kernels. No CUDA or torch types: the host side fills these in
// FP64 and copies them (cast to the kernel's Real) to device memory.
#pragma once

#include <stdint.h>

namespace mcg {

// Face kinds, in the order of montecarlo/boundary.h:137-281.
enum FaceKind { F_SPEC = 0, F_DIFF = 1, F_ISOT = 2, F_PERI = 3, F_INTER = 4 };

// Tally problems (montecarlo/problem.h:157-239): rows 1, 3, 4, and for the
// scatter-count binned CumTemp / CumFlux size + 1 and 3 (size + 1).
enum Problem { P_TEMP = 0, P_FLUX = 1, P_MULTI = 2, P_CUMTEMP = 3, P_CUMFLUX = 4 };

// Row class of field row r: the fixed-point quantum and the checksum it
// uses (time rows of CumTemp all share class 0, the three flux components
// of every CumFlux bin classes 0..2).
__host__ __device__ inline int rowClass(int problem, int r) {
    return problem == P_CUMTEMP ? 0 : (problem == P_CUMFLUX ? r % 3 : r);
}
// number of row classes (checksums) of a problem with `rows` rows
__host__ __device__ inline int rowClasses(int problem, int rows) {
    return problem == P_CUMTEMP ? 1 : (problem == P_CUMFLUX ? 3 : rows);
}

// Reason a phonon stopped (device counters).
enum Counter {
    C_PHONON_STEPS = 0,  // live phonons x dt steps processed
    C_EVENTS,            // completed loop iterations (flight + event)
    C_SCATTERS,          // relaxation-time scatters
    C_ESCAPES,           // numerical escapes / Inter misses
    C_HORIZON,           // alive at the time horizon
    C_MAXSCAT,           // stopped at nscat >= maxscat
    C_MAXLOOP,           // stopped at maxloop iterations
    C_ABSORBED,          // absorbed by an isothermal wall
    C_REPLAY_EXHAUSTED,  // replay stream ran out
    C_BAD,               // non-finite state (killed)
    C_LIVE,              // live phonons written by the last launch
    C_NCOUNTERS = 16
};

// Status bits returned to the host.
enum Status {
    S_OK = 0,
    S_REPLAY_EXHAUSTED = 1,
    S_NONFINITE = 2,
    S_BAD_CELL = 4,
    S_TIMEOUT = 8,  // a bounded device-side wait gave up (results discarded)
};

// One face of a subdomain. A Parallelepiped's face f lies on axis f % 3 of
// its reduced coordinates at u = 0 (f < 3) or u = S (f >= 3). The faces of
// the other shapes (SdomD::gen) are planes in the subdomain's frame
// coordinates: gp[0..2] . u + gp[3] is the signed distance from the face.
//
// An Inter face paired with several others (montecarlo/boundary.cpp:349-359)
// keeps its candidates as entries of its subdomain's continuation slot:
// more = count << 8 | first entry; each candidate entry holds the pair map
// (to, toface, tang, A, b) and, in n[k], the factor that turns the target's
// escape tolerance into frame units along axis k (S_k / height_k).
template <typename R>
struct FaceD {
    int kind;
    int to;       // destination subdomain (Peri / Inter), else -1
    int toface;   // axis face of `to` the phonon arrives on, -1 for none
    int ident;    // 1 if the Peri rotation is the identity
    int tang;     // 1 if the map keeps the tangential cell coordinates
    int more;     // Inter candidates in the continuation slot (see above), 0 for one pair
    R n[3];       // inward unit normal (Spec reflection)
    R rot[9];     // rotation z-hat -> n, row-major (Diff, Isot emission)
    R Rd[9];      // Peri direction rotation, row-major
    R A[9];       // reduced-coordinate map into subdomain `to`: u' = A u + b
    R b[3];
    R T;          // emission temperature after pairing (Isot / Peri)
    R gp[4];      // plane in frame coordinates (general faces)
};

// Faces a subdomain slot holds. A subdomain with more faces, or with Inter
// faces paired several times, also takes the next slot (its continuation):
// faces MAX_FACES .. nface - 1 are the continuation's f[0 ..], followed by
// the Inter candidates.
constexpr int MAX_FACES = 6;

template <typename R>
struct SdomD {
    R Minv[9];    // row-major inverse edge matrix
    R M[9];       // row-major edge matrix
    R o[3];       // origin
    R S[3];       // shape as reals
    R gradT[3];   // volumetric gradient (EmitSubdomain)
    R grot[9];    // rotation z-hat -> gradT-hat
    R eps;        // escape tolerance in path length
    int shape[3];    // walk cells per axis: max(div, 1), or WALK_CELLS on an
                     // axis without tally cells (finer FP32 offsets)
    int tstride[3];  // field column stride of each axis, 0 if the axis has
                     // no tally cells
    int accum;       // Subdomain::accumFlag (montecarlo/subdomain.cpp:47-70)
    int colbeg;      // first field column, -1 if the subdomain has none
    int gen;         // 1: not a Parallelepiped (faces are frame-coordinate
                     // planes, the frame a box around the shape)
    int nface;       // faces in the reference's bdry<I>() order
    FaceD<R> f[MAX_FACES];
};

// Largest number of pieces (sub-triangles of a Polygon face, sub-volumes of
// a Prism or Pyramid) of an emitter.
constexpr int MAX_PIECES = 7;

// Emitter: a volume (face = -1) or a face of a subdomain. Parallelepiped
// emitters (fold < 0) draw in the subdomain's reduced coordinates. The
// others draw a piece (one uniform against thr when npiece > 1), then
// ncoord uniforms c folded per `fold`, and start at u = U0 + L c in the
// subdomain's frame coordinates.
enum { FOLD_NONE = 0, FOLD_PRISM = 1, FOLD_TETRA = 2, FOLD_TRIANGLE = 3 };
struct EmitterD {
    int sdom;
    int face;
    int fold;    // -1 Parallelepiped, else FOLD_*
    int ncoord;  // 2 (faces) or 3 (volumes)
    int npiece;
    int pad;
    unsigned long long thr[MAX_PIECES];  // piece i: first i with word < thr[i]
    double U0[MAX_PIECES][3];
    double L[MAX_PIECES][9];             // row-major
};

// Packed cell: the low 5 bits of the subdomain slot and three 9-bit cell
// indices; the slot's sixth bit rides in bit 26 of the prop word.
constexpr int CELL_BITS = 9;
constexpr int MAX_SHAPE = 1 << CELL_BITS;
constexpr int MAX_SDOM = 64;
// Walk cells on an axis that carries no tally cells (div = 0) of a
// subdomain with a 0-D or 1-D field: positions are stored as cell index +
// offset, so this sets the FP32 resolution along that axis.
constexpr int WALK_CELLS = 256;

// Bytes moved per phonon per launch by the FP32 kernel's state (read once,
// written once): three 16-byte words.
constexpr int STATE_BYTES_F32 = 48;
constexpr int STATE_BYTES_F64 = 80;

}  // namespace mcg
