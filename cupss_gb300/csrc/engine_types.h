// Parameter blocks shared by the host planner and the CUDA kernels.
//
// Spectral storage ("packed half spectrum"): a real field of sx*sy*sz points is
// held as Lx*sy*sz complex values, Lx = sx/2, index ((kz*sy + ky)*Lx + kx').
// Column kx' = 0 packs the two real-in-x planes kx = 0 and kx = sx/2:
//   Z(ky,kz) = F(0,ky,kz) + i F(sx/2,ky,kz),
// so F(0,k) = (Z(k) + conj Z(-k))/2 and F(sx/2,k) = -i (Z(k) - conj Z(-k))/2.
// Columns 0 < kx' < sx/2 hold F(kx',ky,kz); kx > sx/2 follow by Hermitian symmetry.
// This is the same information as the reference's full C2C float2 array after its
// per-step projection onto real fields (src/field.cpp:63-89), in half the bytes.
#pragma once
#if defined(__CUDACC_RTC__)
typedef unsigned int uint32_t;
#else
#include <cstdint>
#include <cuda_runtime.h>
#endif

namespace cupssgb {

constexpr int kMaxXIn = 8;         // real-space inputs of one row pass
constexpr int kMaxProd = 8;        // products per phase
constexpr int kMaxOrder = 8;       // factors per product
constexpr int kMaxPhaseFields = 12;
constexpr int kMaxTerms = 24;
constexpr int kMaxPres = 48;
constexpr int kMaxFields = 32;
constexpr int kMaxSrc = 4;         // prefetched state sources of one field's update

// One q-monomial: pre * q^(2 q2n) * qx^iqx * qy^iqy * qz^iqz * |q|^-invq.
// For explicit terms `pre` already carries the reference's sign rule
// (src/term_init.cpp:151-152); the factor i is applied per term via TermK::s.
struct PresK {
  float pre;
  int q2n, iqx, iqy, iqz, invq;
};

// kTermMerged: a product term whose real-space product the row pass adds into another
// term's channel (same prefactors): its contribution arrives with that term, so the
// update skips it.
enum TermKind : int { kTermSingle = 0, kTermProduct = 1, kTermConst = 2, kTermMerged = 3 };

struct TermK {
  int kind;    // TermKind
  int src;     // prefetch slot of the source state (single) or product slot (product)
  int s;       // 1 -> multiply by i (odd number of iq factors in the first pres)
  int npres, pres0;
};

struct FieldK {
  const float2* cur;     // state at the start of the phase
  float2* next;          // state after the phase (ping-pong partner)
  float2* chan;          // masked, 1/N-scaled inverse along the line axis, or null
  int dynamic, noisy;
  int nterms, term0;
  int nimp, imp0;
  int order;             // dealias order (max product size the field appears in)
  int fid;               // field id used in the noise counter
  float noise_base;      // sqrt(dt/dV*A) (dynamic) or that / sqrt(dt) (non-dynamic)
  int noise_q2n, noise_invq;
  int chan_xlimit;       // last kx' column with unmasked content (sx/(order+1))
  int chan_ylimit;       // |n_y| limit (sy/(order+1)), used to skip empty 3D tiles
  int chan_zlimit;       // |n_z| limit (sz/(order+1))
  int nsrc;              // states prefetched into shared memory for this field
  int src[kMaxSrc];      // their field indices (own state included when read)
  int self_src;          // prefetch slot of the own state, or -1
};

// One member of a batch: a solver can hold several independent systems of the same
// structure and grid, member z at blockIdx.z of every step launch.  Each member has
// its own Philox key, its own step count (the noise counter) and an active flag (an
// inactive member is skipped by every kernel and does not count steps).
struct MemberK {
  uint32_t key0, key1, step, active;
};
// Per-member numerical values of one phase: [k] = pres[k].pre for k < kMaxPres,
// [kMaxPres + fi] = f[fi].noise_base.
constexpr int kMemberVals = kMaxPres + kMaxPhaseFields;

enum LineGeo : int {
  kGeoCol = 0,   // 1D/2D: lines are y-columns, elem = y*Lx + kx'
  kGeoY3 = 1,    // 3D y lines, elem = (z*sy + y)*Lx + kx', blockIdx.y = z
  kGeoZ3 = 2,    // 3D z lines, elem = (z*sy + ky)*Lx + kx', blockIdx.y = ky (or pair)
};

enum LineMode : int { kModeTurn = 0, kModeFwd = 1, kModeInv = 2 };

struct LineParams {
  int sx, sy, sz, Lx, L;
  int geo, mode, W;
  float stepqx, stepqy, stepqz, dt, invN, sqrtN, sqrtHalfN;
  int src_slots;                    // turnaround: shared-memory slots for prefetched states
  int tslot;                        // turnaround: transpose slot of the dealiased-copy inverse
  // products (turnaround) or channels to transform (fwd/inv passes)
  int n_prod;
  const float2* prod_in[kMaxProd];
  float2* prod_out[kMaxProd];       // fwd/inv passes only (may equal prod_in)
  int inv_xlimit[kMaxProd];         // inv pass: skip tiles with kx0 > limit
  int inv_lkeep[kMaxProd];          // inv pass: > 0 -> input positions n with |n| >= inv_lkeep
                                    // (n = k or k - L) are known zero and not read
  int nf;
  FieldK f[kMaxPhaseFields];
  TermK term[kMaxTerms];
  PresK pres[kMaxPres];             // term pres, then implicit pres (raw, unsigned)
  const float2* state[kMaxFields];  // current state of every field
  uint32_t key0, key1, step;
  const float2* tw;
  // members[z]: key, step count and active flag of the system at blockIdx.z (null: key and
  // step above).  Batches: member z's arrays start z * mstride elements after every
  // pointer above and its values are mvals[z] (null for a single system: values above).
  size_t mstride;
  const MemberK* members;
  const float* mvals;               // [member][kMemberVals]
  uint32_t step_off;                // noise step = members[z].step + step_off (steps replayed in one graph)
};

enum XInMode : int { kXInSpectral = 0, kXInReal = 1, kXInRealPair = 2 };   // RealPair: float2 (x, y) reads .x
enum XOutMode : int { kXOutSpectral = 0, kXOutReal = 1, kXOutRealPair = 2 };

struct XParams {
  int Lx, rows;
  int in_mode, out_mode;
  float out_scale;                  // multiplies every product, in real or spectral output
  int n_in;
  const float2* in[kMaxXIn];        // spectral channels (float2) or real rows (as pairs)
  int in_xcols[kMaxXIn];            // spectral inputs: columns kx' >= in_xcols are known zero
                                    // and not read (0: every column is read)
  int n_prod;
  void* out[kMaxProd];
  int prod_n[kMaxProd];
  int prod_f[kMaxProd][kMaxOrder];
  // 1: product q is added to the values of product q - 1 (one output channel, transformed
  // and written once, after its last product); 0: product q starts a channel
  int prod_add[kMaxProd];
  const float2* tw;
  size_t mstride;                   // batches: member z's rows start z * mstride elements on
  const MemberK* members;           // null for a single system
};

// xy-plane pass of a 3D phase (plane.cuh): product of one channel, plane by plane.
struct PlaneParams {
  int nc;             // input columns kx' < nc carry content
  int ykeep;          // input rows with |n_y| >= ykeep are known zero (ykeep > sy/2: every row is read)
  int ps;             // plane-store pitch in float2 (>= max(nc, Lx/C), = 8 mod 16)
  int order;          // power of the real values (product size)
  float out_scale;    // multiplies every product value
  const float2* in;   // H'(kx', ky, z) at ((z*sy + ky)*Lx + kx'): x and y spectral, z positional
  float2* out;        // G''(kx', ky, z), same layout
  const float2* tw;
  size_t mstride;     // batches: member z at blockIdx.z * mstride elements
  const MemberK* members;
};

// Fused launches over several batched solvers of one system structure on different grids
// ("grid classes"): class c owns a contiguous range of blockIdx.x and its members are
// blockIdx.z < span[c].  Passed by value (8 LineParams stay below the 32 KB parameter limit).
constexpr int kMaxClasses = 8;
struct MultiTurnParams {
  LineParams p[kMaxClasses];
  int span[kMaxClasses];
};
struct MultiRowParams {
  XParams x[kMaxClasses];
  int span[kMaxClasses];
};
struct MultiTickParams {
  MemberK* members[kMaxClasses];
  int n[kMaxClasses];
  int nc;
  uint32_t inc;
};

struct ExpandParams {
  int sx, sy, sz, Lx;
  const float2* spec;   // packed half spectrum, fully transformed
  float2* full;         // reference layout, sx*sy*sz complex
};

// Reference-layout full spectrum -> packed half spectrum (Hermitian projection, the
// effect of the reference's IFFT -> real part -> FFT round trip, src/field.cpp:64-89).
struct CompressParams {
  int sx, sy, sz, Lx;
  const float2* full;
  float2* spec;
};

// Dealiased, 1/N-scaled copy of a packed spectrum (kept modes only).
struct MaskParams {
  int sx, sy, sz, Lx;
  int xlim, ylim, zlim;
  float scale;
  const float2* spec;
  float2* out;
};

}  // namespace cupssgb
