// sf_oracle.cpp -- CPU ORACLE for the Starfish ES-PIC/DSMC hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain serial C++ (FP64,
// array-of-structs particles like the reference's `Particle` objects), the
// algorithms of the Java reference for the hot path.  Only the test-suite,
// `__graft_entry__.smoke()` and the CPU-baseline legs of `bench.py` load it,
// and only to check results against and as the CPU baseline.  The product
// (libstarfish_gpu.so) never
// links, loads or calls it.
//
// Parity status: the Java reference cannot be compiled or run here (no JDK)
// and ships no tests, golden vectors or fixtures, so this restatement is
// "parity unpinned" against the reference itself.  It is pinned instead by
// analytic known-answer tests (tests/test_oracle_cpu.py) and by golden
// fixtures generated from it (tests/golden/make_golden.py).
//
// Every function cites the reference file:line it follows (paths relative to
// the Starfish project root, `src/starfish/...`).
//
// Deliberate differences from the Java code (all below FP64 rounding level):
//  * Sparse rows are summed in ascending column order; Java iterates its
//    HashMap rows in hash-bucket order.
//  * Segment candidate sets are visited in node order, not HashSet order
//    (only matters for exact ties between two segments).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ----------------------------------------------------------------------------
// Constants  (src/starfish/core/common/Constants.java:20-34)
// ----------------------------------------------------------------------------
constexpr double EPS0 = 8.85418782e-12;
constexpr double KB = 1.3806503e-23;
constexpr double QE = 1.60217646e-19;
constexpr double AMU = 1.66053886e-27;
constexpr double FLT_EPS = 1e-7;
constexpr double PI = 3.14159265358979323846;
const double SQRT2 = std::sqrt(2.0);

// Enumerations, with the reference's numeric codes.
// NodeType (core/domain/Mesh.java:172-173)
enum { NODE_OPEN = -1, NODE_DIRICHLET = 0, NODE_INSULATOR = 1, NODE_INTERNAL = 2 };
// DomainBoundaryType (core/domain/Mesh.java:140-141)
enum { DB_OPEN = -1, DB_DIRICHLET = 0, DB_NEUMANN = 1, DB_PERIODIC = 2, DB_SYMMETRY = 3,
       DB_MESH = 4, DB_SINK = 5, DB_CIRCUIT = 6 };
// Face (core/domain/Mesh.java:107-108)
enum { F_RIGHT = 0, F_TOP = 1, F_LEFT = 2, F_BOTTOM = 3 };
// Boundary (segment) type (core/boundaries/Boundary.java:124-125)
enum { BT_DIRICHLET = 0, BT_OPEN = 1, BT_SINK = 2, BT_VIRTUAL = 3, BT_INSULATOR = 4 };
// Surface impact handlers (interactions/SurfaceInteraction.java:29-36); PASS = boundary
// without a material (KineticMaterial.java:570-571 skips the interaction).
enum { SURF_PASS = -1, SURF_ABSORB = 0, SURF_NONE = 1, SURF_SPECULAR = 2, SURF_DIFFUSE = 3 };
// Domain type
enum { DOM_XY = 0, DOM_RZ = 1, DOM_ZR = 2 };

// ----------------------------------------------------------------------------
// java.util.Random restated from the Java SE API specification (48-bit LCG).
// Used as Starfish.rnd() (core/common/Starfish.java:238-246).
// ----------------------------------------------------------------------------
struct JRandom {
  uint64_t seed = 0;
  void set_seed(int64_t s) { seed = ((uint64_t)s ^ 0x5DEECE66DULL) & ((1ULL << 48) - 1); }
  int next(int bits) {
    seed = (seed * 0x5DEECE66DULL + 0xBULL) & ((1ULL << 48) - 1);
    return (int)(int64_t)(seed >> (48 - bits));
  }
  double nextDouble() {
    return (double)(((int64_t)next(26) << 27) + next(27)) * 0x1.0p-53;
  }
};

// Samplers (core/common/Utils.java:27-57, 69-87, 121-136; Vec.java:450-471)
double sample_maxw_1d(JRandom& r, double v_th) {
  double sum = 0;
  const int M = 12;
  for (int i = 0; i < M; i++) sum += r.nextDouble();
  double fm = (sum - 0.5 * M) * std::sqrt(12.0 / M);
  return std::sqrt(0.5) * v_th * fm;
}
void sample_maxw_3d(JRandom& r, double v_th, double out[3]) {
  out[0] = (v_th * 1.2) * sample_maxw_1d(r, 1);
  out[1] = (v_th * 1.2) * sample_maxw_1d(r, 1);
  out[2] = (v_th * 1.2) * sample_maxw_1d(r, 1);
}
double sample_maxw_speed(JRandom& r, double v_th) {
  double bin_max = 6 * v_th;
  double a = 4 / (std::sqrt(PI) * v_th * v_th * v_th);
  double fm_max = 4 / (std::sqrt(PI) * v_th) * std::exp(-1.0);
  for (;;) {
    double v = r.nextDouble() * bin_max;
    double fm = a * v * v * std::exp(-v * v / (v_th * v_th));
    if ((fm / fm_max) > r.nextDouble()) return v;
  }
}
void isotropic_vel(JRandom& r, double mag, double v[3]) {
  double theta = 2 * PI * r.nextDouble();
  double R = -1.0 + 2 * r.nextDouble();
  double a = std::sqrt(1 - R * R);
  double amag = (mag > 0) ? mag : -mag;
  v[0] = std::cos(theta) * a * amag;
  v[1] = std::sin(theta) * a * amag;
  v[2] = R * amag;
}
void lambertian_vector(JRandom& r, const double n[3], const double t[3], double vec[3]) {
  const double p[3] = {0, 0, 1};
  double cosphi = std::sqrt(1.0 - r.nextDouble());
  if (cosphi > 0.99999) cosphi = 0.99999;
  double theta_vel = 2 * PI * r.nextDouble();
  double sinphi = std::sqrt(1.0 - cosphi * cosphi);
  double c_tang = std::cos(theta_vel) * sinphi;
  double c_normal = cosphi;
  double c_inplane = std::sin(theta_vel) * sinphi;
  for (int i = 0; i < 3; i++) vec[i] = c_tang * t[i] + c_normal * n[i] + c_inplane * p[i];
}
// Bird's gamma function (core/common/Utils.java:218-236)
double bird_gamma(double X) {
  double A = 1.;
  double Y = X;
  if (Y < 1.0) {
    A = A / Y;
  } else {
    do {
      Y = Y - 1;
      if (Y >= 1.) A = A * Y;
    } while (Y >= 1.);
  }
  return A * (1. - 0.5748646 * Y + 0.9512363 * Y * Y - 0.6998588 * Y * Y * Y +
              0.4245549 * Y * Y * Y * Y - 0.1010678 * Y * Y * Y * Y * Y);
}

// ----------------------------------------------------------------------------
// Uniform mesh (core/domain/UniformMesh.java:139-161, Mesh.java:815-1040)
// Node arrays are j-major: u = j*ni + i (Mesh.IJtoN, Mesh.java:893-897).
// ----------------------------------------------------------------------------
struct Mesh {
  int ni, nj;
  double x0[2], dh[2];
  int domain;
  const int8_t* node_type;   // ni*nj
  const int8_t* face_type;   // 4 x max(ni,nj), indexed [face*nmax + index]
  int nmax;
  int nt(int i, int j) const { return node_type[j * ni + i]; }
  int bt(int face, int index) const { return face_type[face * nmax + index]; }
  void pos(double i, double j, double x[2]) const {
    x[0] = x0[0] + i * dh[0];
    x[1] = x0[1] + j * dh[1];
  }
  void XtoL(const double x[2], double lc[2]) const {
    lc[0] = (x[0] - x0[0]) / dh[0];
    lc[1] = (x[1] - x0[1]) / dh[1];
  }
  double R(double i, double j) const {
    if (domain == DOM_RZ) return x0[0] + i * dh[0];
    if (domain == DOM_ZR) return x0[1] + j * dh[1];
    return 1;
  }
  bool dirichlet(int i, int j) const {  // Mesh.isDirichletNode, Mesh.java:326-328
    int t = nt(i, j);
    return t == NODE_DIRICHLET || t == NODE_INTERNAL;
  }
};

int minmax(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Mesh.controlVolumeLCs (Mesh.java:656-744), single mesh without insulator nodes.
void control_volume_lcs(const Mesh& m, double i0, double j0, double delta, double lcs[4][2]) {
  for (int k = 0; k < 4; k++) {
    double i = -1, j = -1;
    switch (k) {
      case 0: i = i0 - delta; j = j0 - delta; break;
      case 1: i = i0 + delta; j = j0 - delta; break;
      case 2: i = i0 + delta; j = j0 + delta; break;
      case 3: i = i0 - delta; j = j0 + delta; break;
    }
    if (i < 0 && m.bt(F_LEFT, minmax((int)(j0 + 0.5), 0, m.nj - 1)) != DB_MESH) i = 0;
    if (i > m.ni - 1 && m.bt(F_RIGHT, minmax((int)(j0 + 0.5), 0, m.nj - 1)) != DB_MESH) i = m.ni - 1;
    if (j < 0 && m.bt(F_BOTTOM, minmax((int)(i0 + 0.5), 0, m.ni - 1)) != DB_MESH) j = 0;
    if (j > m.nj - 1 && m.bt(F_TOP, minmax((int)(i0 + 0.5), 0, m.ni - 1)) != DB_MESH) j = m.nj - 1;
    if (i < 0 || j < 0 || i > m.ni - 1 || j > m.nj - 1) {  // no neighbour mesh exists
      if (i < 0) i = 0;
      if (j < 0) j = 0;
      if (i >= m.ni - 1) i = m.ni - 1;
      if (j >= m.nj - 1) j = m.nj - 1;
    }
    lcs[k][0] = i;
    lcs[k][1] = j;
  }
  lcs[0][1] = std::max(lcs[0][1], lcs[1][1]);
  lcs[1][1] = lcs[0][1];
  lcs[1][0] = std::min(lcs[1][0], lcs[2][0]);
  lcs[2][0] = lcs[1][0];
  lcs[1][0] = std::min(lcs[1][0], lcs[2][0]);  // repeated as in the reference
  lcs[2][0] = lcs[1][0];
  lcs[2][1] = std::max(lcs[2][1], lcs[3][1]);
  lcs[3][1] = lcs[2][1];
  lcs[3][0] = std::max(lcs[3][0], lcs[0][0]);
  lcs[0][0] = lcs[3][0];
}

// Mesh.area (Mesh.java:961-985): two-triangle area of the control volume.
double cv_area(const Mesh& m, double i0, double j0) {
  double lcs[4][2], V[4][2];
  control_volume_lcs(m, i0, j0, 0.5, lcs);
  for (int k = 0; k < 4; k++) m.pos(lcs[k][0], lcs[k][1], V[k]);
  double A = 0.5 * std::fabs(V[0][0] * V[1][1] - V[0][0] * V[2][1] + V[1][0] * V[2][1] -
                             V[1][0] * V[0][1] + V[2][0] * V[0][1] - V[2][0] * V[1][1]);
  A += 0.5 * std::fabs(V[0][0] * V[2][1] - V[0][0] * V[3][1] + V[2][0] * V[3][1] -
                       V[2][0] * V[0][1] + V[3][0] * V[0][1] - V[3][0] * V[2][1]);
  return A;
}

// Mesh.nodeVol (Mesh.java:998-1020)
double node_vol(const Mesh& m, double i0, double j0) {
  if (m.domain == DOM_XY) return 1.0 * cv_area(m, i0, j0);
  double r = m.R(i0, j0);
  if (m.domain == DOM_RZ) {
    if (i0 == 0) r = m.R(i0 + 0.25, j0);
    else if (i0 == m.ni - 1) r = m.R(i0 - 0.25, j0);
  } else if (m.domain == DOM_ZR) {
    if (j0 == 0) r = m.R(i0, j0 + 0.25);
    else if (j0 == m.nj - 1) r = m.R(i0, j0 - 0.25);
  }
  return 2 * PI * cv_area(m, i0, j0) * r;
}

// ----------------------------------------------------------------------------
// Field2D gather / scatter (core/domain/Field2D.java:244-390)
// ----------------------------------------------------------------------------
double gather_safe(const Mesh& m, const double* f, double fi, double fj) {
  int i = (int)fi, j = (int)fj;
  double di = fi - i, dj = fj - j;
  if (i < 0) { i = 0; di = 0; }
  if (j < 0) { j = 0; dj = 0; }
  if (i >= m.ni - 1) { i = m.ni - 1; di = 0; }
  if (j >= m.nj - 1) { j = m.nj - 1; dj = 0; }
  const int ni = m.ni;
  double v = (1 - di) * (1 - dj) * f[j * ni + i];
  if (di > 0) v += di * (1 - dj) * f[j * ni + i + 1];
  if (di > 0 && dj > 0) v += di * dj * f[(j + 1) * ni + i + 1];
  if (dj > 0) v += (1 - di) * dj * f[(j + 1) * ni + i];
  return v;
}
// Field2D.gather(double[]) falls back to gather_safe on an out-of-range index
// (Field2D.java:302-309, 318-350).
double gather(const Mesh& m, const double* f, const double lc[2]) {
  int i = (int)lc[0], j = (int)lc[1];
  if (i < 0 || j < 0 || i + 1 > m.ni - 1 || j + 1 > m.nj - 1) return gather_safe(m, f, lc[0], lc[1]);
  double di = lc[0] - i, dj = lc[1] - j;
  const int ni = m.ni;
  double v = (1 - di) * (1 - dj) * f[j * ni + i];
  v += di * (1 - dj) * f[j * ni + i + 1];
  v += di * dj * f[(j + 1) * ni + i + 1];
  v += (1 - di) * dj * f[(j + 1) * ni + i];
  return v;
}
// Field2D.scatter (Field2D.java:244-295) including the Ruyten RZ/ZR weights.
void scatter(const Mesh& m, double* f, double fi, double fj, double val) {
  int i = (int)fi, j = (int)fj;
  double di = fi - i, dj = fj - j;
  if (i < 0 || j < 0 || i >= m.ni - 1 || j >= m.nj - 1) return;
  if (m.domain == DOM_RZ) {
    double rp = m.R(i + 1, fj), rm = m.R(i, fj), r = m.R(fi, fj);
    di = 1 - (0.5 * (rp - r) * (2 * rp + 3 * rm - r) / (rp * rp - rm * rm));
  } else if (m.domain == DOM_ZR) {
    double rp = m.R(fi, j + 1), rm = m.R(fi, j), r = m.R(fi, fj);
    di = fi - i;
    dj = 1 - (0.5 * (rp - r) * (2 * rp + 3 * rm - r) / (rp * rp - rm * rm));
  }
  const int ni = m.ni;
  f[j * ni + i] += (1 - di) * (1 - dj) * val;
  f[j * ni + i + 1] += di * (1 - dj) * val;
  f[(j + 1) * ni + i + 1] += di * dj * val;
  f[(j + 1) * ni + i] += (1 - di) * dj * val;
}

// ----------------------------------------------------------------------------
// Boundary segments (core/boundaries/LinearSegment.java:22-46, 113-179)
// ----------------------------------------------------------------------------
struct Seg {
  double x1[2], x2[2];
  double normal[3], tangent[3];
  int btype;     // Boundary type of the owning boundary
  int model;     // surface impact handler of (boundary material, species)
  double vth;    // boundary thermal speed for DIFFUSE (Boundary.getVth)
  double c_rest, c_accom;
};
void seg_init(Seg& s) {
  double dx = s.x2[0] - s.x1[0], dy = s.x2[1] - s.x1[1];
  double len = std::sqrt(dx * dx + dy * dy);
  dx /= len;
  dy /= len;
  s.tangent[0] = dx; s.tangent[1] = dy; s.tangent[2] = 0;
  s.normal[0] = -dy; s.normal[1] = dx; s.normal[2] = 0;
}
bool infinite_line_intersect(const double p1[2], const double p2[2], const double p3[2],
                             const double p4[2], double xp[2]) {
  double x1 = p1[0], x2 = p2[0], x3 = p3[0], x4 = p4[0];
  double y1 = p1[1], y2 = p2[1], y3 = p3[1], y4 = p4[1];
  double den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
  if (den == 0) return false;
  xp[0] = ((x1 * y2 - y1 * x2) * (x3 - x4) - (x1 - x2) * (x3 * y4 - y3 * x4)) / den;
  xp[1] = ((x1 * y2 - y1 * x2) * (y3 - y4) - (y1 - y2) * (x3 * y4 - y3 * x4)) / den;
  return true;
}
void seg_intersect(const Seg& s, const double p3[2], const double p4[2], double t[2]) {
  const double* p1 = s.x1;
  const double* p2 = s.x2;
  double xp[2];
  if (!infinite_line_intersect(p1, p2, p3, p4, xp)) { t[0] = -1; t[1] = -1; return; }
  if (std::fabs(p2[0] - p1[0]) > 1e-6) t[0] = (xp[0] - p1[0]) / (p2[0] - p1[0]);
  else t[0] = (xp[1] - p1[1]) / (p2[1] - p1[1]);
  if (t[0] < -FLT_EPS || t[0] > (1 + FLT_EPS)) { t[0] = -1; t[1] = -1; return; }
  if (std::fabs(p4[0] - p3[0]) > 1e-6) t[1] = (xp[0] - p3[0]) / (p4[0] - p3[0]);
  else t[1] = (xp[1] - p3[1]) / (p4[1] - p3[1]);
  if (t[1] < -FLT_EPS || t[1] > (1 + FLT_EPS)) { t[0] = -1; t[1] = -1; return; }
  if (t[0] < 0) t[0] = 0;
  if (t[1] < 0) t[1] = 0;
  if (t[0] > 1) t[0] = 1;
  if (t[1] > 1) t[1] = 1;
}
bool in_box(const double x[2], const double b1[2], const double b2[2]) {
  return x[0] >= b1[0] && x[0] <= b2[0] && x[1] >= b1[1] && x[1] <= b2[1];
}
// Segment.segmentInBox (core/boundaries/Segment.java:246-300)
bool segment_in_box(const Seg& s, const double b1[2], const double b2[2]) {
  if (in_box(s.x1, b1, b2) || in_box(s.x2, b1, b2)) return true;
  for (int face = 0; face < 4; face++) {
    double f1[2], f2[2];
    switch (face) {
      case 0: f1[0] = b1[0]; f1[1] = b1[1]; f2[0] = b2[0]; f2[1] = b1[1]; break;  // bottom
      case 1: f1[0] = b2[0]; f1[1] = b1[1]; f2[0] = b2[0]; f2[1] = b2[1]; break;  // right
      case 2: f1[0] = b2[0]; f1[1] = b2[1]; f2[0] = b1[0]; f2[1] = b2[1]; break;  // top
      default: f1[0] = b1[0]; f1[1] = b2[1]; f2[0] = b1[0]; f2[1] = b1[1]; break; // left
    }
    double t[2];
    seg_intersect(s, f1, f2, t);
    if (t[0] >= 0) return true;
  }
  return false;
}

// ----------------------------------------------------------------------------
// Particle push (core/materials/KineticMaterial.java:299-422, 424-462, 471-750)
// ----------------------------------------------------------------------------
struct Particle {  // 12 doubles, layout shared with the Python side
  double pos[3], vel[3], lc[2], dt, mpw, alive, spare;
};
static_assert(sizeof(Particle) == 12 * sizeof(double), "particle layout");

struct PushCtx {
  const Mesh* m;
  const double* efi;
  const double* efj;
  double qm;       // q/m
  double mass, charge;
  double dt;
  const Seg* segs;
  const int* node_seg_ptr;  // ni*nj+1
  const int* node_seg_idx;
  // surface accumulators: per segment, split linearly over the segment ends
  // (Material.addSurfaceMomentum / addSurfaceMassDeposit, Material.java:759-796)
  double* flux;     // 2*nseg
  double* deposit;  // 2*nseg
  double boundary_charge;
  JRandom* rnd;
};

void mirror(double vec[3], const double r[3]) {  // Vec.mirror (Vec.java:406-418)
  double t_mag = vec[0] * r[0] + vec[1] * r[1] + vec[2] * r[2];
  double t[3] = {r[0] * t_mag, r[1] * t_mag, r[2] * t_mag};
  for (int k = 0; k < 3; k++) vec[k] = -t[k] + (vec[k] - t[k]);
}

// Material.performSurfaceInteraction with a single handler of probability 1
// (Material.java:279-336) and SurfaceInteraction handlers (SurfaceInteraction.java:84-213).
bool surface_interaction(PushCtx& c, const Seg& s, double vel[3]) {
  switch (s.model) {
    case SURF_ABSORB: return false;
    case SURF_NONE: return true;
    case SURF_SPECULAR: {
      double mag = std::sqrt(vel[0] * vel[0] + vel[1] * vel[1]) * SQRT2;
      vel[0] += s.normal[0] * mag;
      vel[1] += s.normal[1] * mag;
      return true;
    }
    case SURF_DIFFUSE: {
      double v_refl = std::sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]) * s.c_rest;
      double v_diff = sample_maxw_speed(*c.rnd, s.vth);
      double v_mag = v_refl + s.c_accom * (v_diff - v_refl);
      double dir[3];
      lambertian_vector(*c.rnd, s.normal, s.tangent, dir);
      for (int k = 0; k < 3; k++) vel[k] = v_mag * dir[k];
      return true;
    }
  }
  return false;
}

bool process_boundary(PushCtx& c, Particle& p, const double old[2], const double lc_old[2]) {
  const Mesh& m = *c.m;
  double dt0 = p.dt;
  p.dt = 0;
  double lc_min[2] = {std::min(p.lc[0], lc_old[0]), std::min(p.lc[1], lc_old[1])};
  double lc_max[2] = {std::max(p.lc[0], lc_old[0]), std::max(p.lc[1], lc_old[1])};
  int i_min = (int)lc_min[0], i_max = (int)lc_max[0];
  int j_min = (int)lc_min[1], j_max = (int)lc_max[1];
  if (i_min < 0) i_min = 0;
  if (j_min < 0) j_min = 0;
  if (i_max >= m.ni) i_max = m.ni - 1;
  if (j_max >= m.nj) j_max = m.nj - 1;

  double tp_min = 2.0, tsurf_min = 0;
  int seg_min = -1;
  // candidate set: DIRICHLET/SINK segments listed on the nodes of the box
  std::vector<int> cand;
  for (int i = i_min; i <= i_max; i++)
    for (int j = j_min; j <= j_max; j++) {
      int u = j * m.ni + i;
      for (int k = c.node_seg_ptr[u]; k < c.node_seg_ptr[u + 1]; k++) {
        int s = c.node_seg_idx[k];
        int bt = c.segs[s].btype;
        if (bt == BT_DIRICHLET || bt == BT_SINK)
          if (std::find(cand.begin(), cand.end(), s) == cand.end()) cand.push_back(s);
      }
    }
  for (int s : cand) {
    const Seg& seg = c.segs[s];
    double t[2];
    seg_intersect(seg, old, p.pos, t);
    double t_part = t[1];
    if (t_part > 0) {
      double vmag2 = std::sqrt(p.vel[0] * p.vel[0] + p.vel[1] * p.vel[1]);
      double acos = (seg.normal[0] * p.vel[0] + seg.normal[1] * p.vel[1]) / vmag2;
      if (t_part < FLT_EPS && (acos > 0 || seg.btype == BT_VIRTUAL)) continue;
      if (t_part < tp_min) {
        tp_min = t_part;
        tsurf_min = t[0];
        seg_min = s;
      }
    }
  }
  bool alive = true;
  if (seg_min >= 0) {
    const Seg& seg = c.segs[seg_min];
    tp_min *= 0.9999;
    p.pos[0] = old[0] + tp_min * (p.pos[0] - old[0]);
    p.pos[1] = old[1] + tp_min * (p.pos[1] - old[1]);
    m.XtoL(p.pos, p.lc);
    p.dt = dt0 * (1 - tp_min);
    if (p.lc[0] < 0 && p.lc[0] > -FLT_EPS) p.lc[0] = 0;
    if (p.lc[1] < 0 && p.lc[1] > -FLT_EPS) p.lc[1] = 0;
    if (seg.model != SURF_PASS) alive = surface_interaction(c, seg, p.vel);
    if (!alive) c.boundary_charge += p.mpw * c.charge;
    if (seg.btype == BT_SINK) alive = false;
    c.flux[2 * seg_min] += p.mpw * (1 - tsurf_min);
    c.flux[2 * seg_min + 1] += p.mpw * tsurf_min;
    if (!alive) {
      c.deposit[2 * seg_min] += p.mpw * (1 - tsurf_min);
      c.deposit[2 * seg_min + 1] += p.mpw * tsurf_min;
      return alive;
    }
  }
  if (p.lc[0] < 0 || p.lc[1] < 0 || p.lc[0] >= m.ni - 1 || p.lc[1] >= m.nj - 1) {
    double t_right = 99, t_top = 99, t_left = 99, t_bottom = 99;
    if (p.lc[0] >= m.ni - 1) t_right = (m.ni - 1.0 - lc_old[0]) / (p.lc[0] - lc_old[0]);
    if (p.lc[1] >= m.nj - 1) t_top = (m.nj - 1.0 - lc_old[1]) / (p.lc[1] - lc_old[1]);
    if (p.lc[0] < 0) t_left = lc_old[0] / (lc_old[0] - p.lc[0]);
    if (p.lc[1] < 0) t_bottom = lc_old[1] / (lc_old[1] - p.lc[1]);
    int exit_face = F_RIGHT;
    double t = t_right;
    if (t_top < t) { exit_face = F_TOP; t = t_top; }
    if (t_left < t) { exit_face = F_LEFT; t = t_left; }
    if (t_bottom < t) { exit_face = F_BOTTOM; t = t_bottom; }
    p.lc[0] = lc_old[0] + t * (p.lc[0] - lc_old[0]);
    p.lc[1] = lc_old[1] + t * (p.lc[1] - lc_old[1]);
    if (p.lc[0] < 0) p.lc[0] = 0;
    else if (p.lc[0] > m.ni - 1) p.lc[0] = m.ni - 1;
    if (p.lc[1] < 0) p.lc[1] = 0;
    else if (p.lc[1] > m.nj - 1) p.lc[1] = m.nj - 1;
    double x[2];
    m.pos(p.lc[0], p.lc[1], x);
    p.pos[0] = x[0];
    p.pos[1] = x[1];
    p.dt = dt0 * (1 - t);
    int i = (int)p.lc[0], j = (int)p.lc[1];
    if (exit_face == F_TOP) j++;
    if (exit_face == F_RIGHT) i++;
    if (i < 0) i = 0;
    if (j < 0) j = 0;
    if (i >= m.ni - 1) i = m.ni - 1;
    if (j >= m.nj - 1) j = m.nj - 1;
    int type = (exit_face == F_LEFT || exit_face == F_RIGHT) ? m.bt(exit_face, j) : m.bt(exit_face, i);
    switch (type) {
      case DB_OPEN: return false;
      case DB_SYMMETRY: {  // UniformMesh.faceNormal (UniformMesh.java:176-189)
        double n[3] = {0, 0, 0};
        if (exit_face == F_LEFT) n[0] = 1;
        else if (exit_face == F_RIGHT) n[0] = -1;
        else if (exit_face == F_BOTTOM) n[1] = 1;
        else n[1] = -1;
        mirror(p.vel, n);
        return true;
      }
      case DB_PERIODIC: {
        double xd0 = m.x0[0] + (m.ni - 1) * m.dh[0], xd1 = m.x0[1] + (m.nj - 1) * m.dh[1];
        if (exit_face == F_LEFT) p.pos[0] += (xd0 - m.x0[0]);
        else if (exit_face == F_RIGHT) p.pos[0] -= (xd0 - m.x0[0]);
        else if (exit_face == F_BOTTOM) p.pos[1] += (xd1 - m.x0[1]);
        else p.pos[1] -= (xd1 - m.x0[1]);
        return true;
      }
      default: return false;  // DIRICHLET, NEUMANN, SINK, MESH (single mesh), CIRCUIT (not modelled)
    }
  }
  return true;
}

void rotate_to_rz(Particle& p) {  // KineticMaterial.java:424-442
  double A = p.vel[2] * p.dt, B = p.pos[0];
  double R = std::sqrt(A * A + B * B);
  double cs = B / R, sn = A / R;
  p.pos[2] -= std::asin(sn);
  double v1 = p.vel[0], v2 = p.vel[2];
  p.pos[0] = R;
  p.vel[0] = cs * v1 + sn * v2;
  p.vel[2] = -sn * v1 + cs * v2;
}
void rotate_to_zr(Particle& p) {  // KineticMaterial.java:444-462
  double A = p.vel[2] * p.dt, B = p.pos[1];
  double R = std::sqrt(A * A + B * B);
  double cs = B / R, sn = A / R;
  p.pos[2] += std::acos(cs);
  double v1 = p.vel[1], v2 = p.vel[2];
  p.pos[1] = R;
  p.vel[1] = cs * v1 + sn * v2;
  p.vel[2] = -sn * v1 + cs * v2;
}

// One ParticleMover pass over one particle (KineticMaterial.java:312-416).
// Returns 1 if the particle is alive after the step.
int push_one(PushCtx& c, Particle& p, double stats[5]) {
  const Mesh& m = *c.m;
  if (p.mpw <= 0) { p.alive = 0; return 0; }
  p.dt += c.dt;
  double ef0 = gather(m, c.efi, p.lc);
  double ef1 = gather(m, c.efj, p.lc);
  p.vel[0] += c.qm * ef0 * p.dt;
  p.vel[1] += c.qm * ef1 * p.dt;
  int bounces = 0;
  bool alive = true;
  while (p.dt > 0 && bounces++ < 10) {
    double old[2] = {p.pos[0], p.pos[1]};
    double old_lc[2] = {p.lc[0], p.lc[1]};
    p.pos[0] += p.vel[0] * p.dt;
    p.pos[1] += p.vel[1] * p.dt;
    if (m.domain == DOM_RZ) rotate_to_rz(p);
    else if (m.domain == DOM_ZR) rotate_to_zr(p);
    else p.pos[2] += p.vel[2] * p.dt;
    m.XtoL(p.pos, p.lc);
    alive = process_boundary(c, p, old, old_lc);
    if (!alive) break;
  }
  p.alive = alive ? 1 : 0;
  if (alive) {
    stats[0] += p.mpw;
    stats[1] += p.mpw * p.vel[0];
    stats[2] += p.mpw * p.vel[1];
    stats[3] += p.mpw * p.vel[2];
    stats[4] += p.mpw * std::sqrt(p.vel[0] * p.vel[0] + p.vel[1] * p.vel[1] + p.vel[2] * p.vel[2]);
  }
  return alive ? 1 : 0;
}

Mesh make_mesh(int ni, int nj, const double* x0, const double* dh, int domain,
               const int8_t* node_type, const int8_t* face_type) {
  Mesh m;
  m.ni = ni; m.nj = nj;
  m.x0[0] = x0[0]; m.x0[1] = x0[1];
  m.dh[0] = dh[0]; m.dh[1] = dh[1];
  m.domain = domain;
  m.node_type = node_type;
  m.face_type = face_type;
  m.nmax = std::max(ni, nj);
  return m;
}

// ----------------------------------------------------------------------------
// FVM assembly (core/solver/Solver.java:204-256, 451-726; Mesh.NodeIndexOffset 1164-1196)
// Sparse rows: ordered maps col -> value.
// ----------------------------------------------------------------------------
typedef std::map<int, double> Row;

void node_index_offset(const Mesh& m, double im, double jm, double di, double dj, int ii[2]) {
  double i = im + di, j = jm + dj;
  double fi = i - (int)i, fj = j - (int)j;
  ii[0] = (fi != 0) ? (int)im : (int)i;
  ii[1] = (fj != 0) ? (int)jm : (int)j;
  if (ii[0] < 0 && m.bt(F_LEFT, minmax(ii[1], 0, m.nj - 1)) != DB_MESH) ii[0] = 0;
  if (ii[1] < 0 && m.bt(F_BOTTOM, minmax(ii[0], 0, m.ni - 1)) != DB_MESH) ii[1] = 0;
  if (ii[0] >= m.ni && m.bt(F_RIGHT, minmax(ii[1], 0, m.nj - 1)) != DB_MESH) ii[0] = m.ni - 1;
  if (ii[1] >= m.nj && m.bt(F_TOP, minmax(ii[0], 0, m.ni - 1)) != DB_MESH) ii[1] = m.nj - 1;
}

struct Edge {
  double im, jm, ndl_i, ndl_j;
  int ij[4][2];
};
// Solver.ComputeEdgeData (Solver.java:636-726), faces in Face order RIGHT, TOP, LEFT, BOTTOM.
void compute_edge_data(const Mesh& m, double i0, double j0, Edge e[4]) {
  double lcs[4][2];
  control_volume_lcs(m, i0, j0, 0.5, lcs);
  for (int face = 0; face < 4; face++) {
    int v1 = 0;
    double im = 0, jm = 0;
    switch (face) {
      case F_BOTTOM: v1 = 0; im = i0; jm = j0 - 0.5; break;
      case F_RIGHT: v1 = 1; im = i0 + 0.5; jm = j0; break;
      case F_TOP: v1 = 2; im = i0; jm = j0 + 0.5; break;
      case F_LEFT: v1 = 3; im = i0 - 0.5; jm = j0; break;
    }
    int v2 = v1 + 1;
    if (v2 > 3) v2 = 0;
    if (im < lcs[0][0]) im = lcs[0][0];
    if (im < lcs[3][0]) im = lcs[3][0];
    if (im > lcs[1][0]) im = lcs[1][0];
    if (im > lcs[2][0]) im = lcs[2][0];
    if (jm < lcs[0][1]) jm = lcs[0][1];
    if (jm < lcs[1][1]) jm = lcs[1][1];
    if (jm > lcs[2][1]) jm = lcs[2][1];
    if (jm > lcs[3][1]) jm = lcs[3][1];
    double x1[2], x2[2];
    m.pos(lcs[v1][0], lcs[v1][1], x1);
    m.pos(lcs[v2][0], lcs[v2][1], x2);
    Edge& E = e[face];
    E.ndl_i = x2[1] - x1[1];
    E.ndl_j = -(x2[0] - x1[0]);
    node_index_offset(m, im, jm, -0.5, -0.5, E.ij[0]);
    node_index_offset(m, im, jm, 0.5, -0.5, E.ij[1]);
    node_index_offset(m, im, jm, 0.5, 0.5, E.ij[2]);
    node_index_offset(m, im, jm, -0.5, 0.5, E.ij[3]);
    E.im = im;
    E.jm = jm;
  }
}

struct Gradient {
  int u[6];
  double Gi[6], Gj[6];
  double R;
};
// Solver.getNodeGradient (Solver.java:559-611)
Gradient node_gradient(const Mesh& m, double i, double j) {
  Gradient G;
  for (int k = 0; k < 6; k++) { G.u[k] = -1; G.Gi[k] = 0; G.Gj[k] = 0; }
  Edge e[4];
  compute_edge_data(m, i, j, e);
  for (int f = 0; f < 4; f++) {
    for (int n = 0; n < 4; n++) {
      for (int k = 0; k < 6; k++) {
        int u = e[f].ij[n][1] * m.ni + e[f].ij[n][0];
        if (u == G.u[k] || G.u[k] < 0) {
          G.u[k] = u;
          G.Gi[k] += 0.25 * e[f].ndl_i;
          G.Gj[k] += 0.25 * e[f].ndl_j;
          break;
        }
      }
    }
  }
  double A = cv_area(m, i, j);
  for (int k = 0; k < 6; k++) { G.Gi[k] *= 1 / A; G.Gj[k] *= 1 / A; }
  G.R = m.R(i, j);
  return G;
}

struct Operator {
  std::vector<Row> A, Gi, Gj;
  std::vector<uint8_t> fixed;
};

// Solver.initCoefficients + setNodeFVMCoefficients (Solver.java:204-256, 451-553)
void assemble(const Mesh& m, Operator& op) {
  int nu = m.ni * m.nj;
  op.A.assign(nu, Row());
  op.Gi.assign(nu, Row());
  op.Gj.assign(nu, Row());
  op.fixed.assign(nu, 0);
  for (int j = 0; j < m.nj; j++)
    for (int i = 0; i < m.ni; i++) {
      Gradient G = node_gradient(m, i, j);
      int u = j * m.ni + i;
      for (int v = 0; v < 6 && G.u[v] >= 0; v++) {
        if (G.Gi[v] != 0) op.Gi[u][G.u[v]] += G.Gi[v];
        if (G.Gj[v] != 0) op.Gj[u][G.u[v]] += G.Gj[v];
      }
    }
  for (int i = 0; i < m.ni; i++)
    for (int j = 0; j < m.nj; j++) {
      int u = j * m.ni + i;
      if (m.dirichlet(i, j)) {
        op.A[u].clear();
        op.A[u][u] = 1;
        op.fixed[u] = 1;
        continue;
      }
      if ((i == 0 && m.bt(F_LEFT, j) != DB_MESH) || (i == m.ni - 1 && m.bt(F_RIGHT, j) != DB_MESH)) {
        op.A[u] = op.Gi[u];
        continue;
      }
      if ((j == 0 && m.bt(F_BOTTOM, i) != DB_MESH) || (j == m.nj - 1 && m.bt(F_TOP, i) != DB_MESH)) {
        op.A[u] = op.Gj[u];
        continue;
      }
      Edge e[4];
      compute_edge_data(m, i, j, e);
      for (int f = 0; f < 4; f++) {
        Gradient G = node_gradient(m, e[f].im, e[f].jm);
        double R = G.R;
        for (int k = 0; k < 6; k++) {
          G.Gi[k] *= e[f].ndl_i * R;
          G.Gj[k] *= e[f].ndl_j * R;
        }
        for (int v = 0; v < 6 && G.u[v] >= 0; v++) {
          double val = G.Gj[v] + G.Gi[v];
          if (val != 0) op.A[u][G.u[v]] += val;
        }
      }
      double V = node_vol(m, i, j);
      for (auto& kv : op.A[u]) kv.second *= 1.0 / V;
    }
}

double row_mult(const Row& r, const double* x) {
  double s = 0;
  for (auto& kv : r) s += kv.second * x[kv.first];
  return s;
}

// LinearSolverGS.solve in serial (LinearSolverGS.java:28-67, 74-152): SOR with w=1.4,
// residual ||Ax-b||_2 / N checked every 25 iterations before the sweep.
int gs_solve(const std::vector<Row>& A, double* x, const double* b, int n, int max_it, double tol,
             double* out_norm) {
  // rows flattened once (same values and column order as the sparse rows)
  std::vector<int> ptr(n + 1, 0), col;
  std::vector<double> val, diag(n, 0.0);
  for (int u = 0; u < n; u++) {
    for (auto& kv : A[u]) {
      col.push_back(kv.first);
      val.push_back(kv.second);
      if (kv.first == u) diag[u] = kv.second;
    }
    ptr[u + 1] = (int)col.size();
  }
  int it = 1;
  double norm = 1e66;
  while (it <= max_it) {
    if (it % 25 == 0) {
      double s = 0;
      for (int u = 0; u < n; u++) {
        double r = 0;
        for (int k = ptr[u]; k < ptr[u + 1]; k++) r += val[k] * x[col[k]];
        r -= b[u];
        s += r * r;
      }
      norm = std::sqrt(s) / n;
      if (norm < tol) break;
    }
    for (int u = 0; u < n; u++) {
      double tau = 0;
      for (int k = ptr[u]; k < ptr[u + 1]; k++)
        if (col[k] != u) tau += val[k] * x[col[k]];
      if (std::fabs(diag[u]) < 1e-8) continue;
      double g = (b[u] - tau) / diag[u];
      x[u] = x[u] + 1.4 * (g - x[u]);
    }
    it++;
  }
  it--;
  if (out_norm) *out_norm = norm;
  return it;
}

}  // namespace

// ============================================================================
// C ABI of the oracle (ctypes).  Arrays are j-major node arrays unless noted.
// ============================================================================
extern "C" {

// --- java.util.Random ------------------------------------------------------
void orc_jrandom_doubles(int64_t seed, int n, double* out) {
  JRandom r;
  r.set_seed(seed);
  for (int i = 0; i < n; i++) out[i] = r.nextDouble();
}
void orc_sample_maxw3d(int64_t seed, int n, double v_th, double* out3) {
  JRandom r;
  r.set_seed(seed);
  for (int i = 0; i < n; i++) sample_maxw_3d(r, v_th, out3 + 3 * i);
}
void orc_sample_maxw_speed(int64_t seed, int n, double v_th, double* out) {
  JRandom r;
  r.set_seed(seed);
  for (int i = 0; i < n; i++) out[i] = sample_maxw_speed(r, v_th);
}
double orc_bird_gamma(double x) { return bird_gamma(x); }

// --- mesh set-up ------------------------------------------------------------
// face_type: 4 x max(ni,nj) codes, rows in Face order RIGHT, TOP, LEFT, BOTTOM.
void orc_node_volumes(int ni, int nj, const double* x0, const double* dh, int domain,
                      const int8_t* node_type, const int8_t* face_type, double* vol) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  for (int j = 0; j < nj; j++)
    for (int i = 0; i < ni; i++) vol[j * ni + i] = node_vol(m, i, j);
}
void orc_cell_volumes(int ni, int nj, const double* x0, const double* dh, int domain,
                      const int8_t* node_type, const int8_t* face_type, double* vol) {
  // Mesh.cellVol (Mesh.java:1038-1040)
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  for (int j = 0; j < nj - 1; j++)
    for (int i = 0; i < ni - 1; i++) vol[j * (ni - 1) + i] = node_vol(m, i + 0.5, j + 0.5);
}

// Mesh.setNodeControlVolumes (Mesh.java:1217-1296): node -> segment lists.
// seg_xy: 4 doubles per segment.  Returns the number of (node, segment) entries;
// call with idx == NULL to size the buffer.
int orc_node_segments(int ni, int nj, const double* x0, const double* dh, int nseg,
                      const double* seg_xy, int* ptr, int* idx) {
  std::vector<std::vector<int>> lists(ni * nj);
  for (int s = 0; s < nseg; s++) {
    Seg sg;
    sg.x1[0] = seg_xy[4 * s]; sg.x1[1] = seg_xy[4 * s + 1];
    sg.x2[0] = seg_xy[4 * s + 2]; sg.x2[1] = seg_xy[4 * s + 3];
    double bmin[2] = {std::min(sg.x1[0], sg.x2[0]), std::min(sg.x1[1], sg.x2[1])};
    double bmax[2] = {std::max(sg.x1[0], sg.x2[0]), std::max(sg.x1[1], sg.x2[1])};
    int lcm[2] = {(int)((bmin[0] - x0[0]) / dh[0]), (int)((bmin[1] - x0[1]) / dh[1])};
    int lcp[2] = {(int)((bmax[0] - x0[0]) / dh[0]), (int)((bmax[1] - x0[1]) / dh[1])};
    lcm[0]--; lcm[1]--;
    lcp[0] += 2; lcp[1] += 2;
    if (lcm[0] < 0) lcm[0] = 0;
    if (lcm[1] < 0) lcm[1] = 0;
    if (lcp[0] > ni - 1) lcp[0] = ni - 1;
    if (lcp[1] > nj - 1) lcp[1] = nj - 1;
    for (int j = lcm[1]; j <= lcp[1]; j++)
      for (int i = lcm[0]; i <= lcp[0]; i++) {
        const double bsize = 1.01;
        double b1[2] = {x0[0] + (i - bsize) * dh[0], x0[1] + (j - bsize) * dh[1]};
        double b2[2] = {x0[0] + (i + bsize) * dh[0], x0[1] + (j + bsize) * dh[1]};
        if (!segment_in_box(sg, b1, b2)) continue;
        auto& L = lists[j * ni + i];
        if (std::find(L.begin(), L.end(), s) == L.end()) L.push_back(s);
      }
  }
  int n = 0;
  for (int u = 0; u < ni * nj; u++) {
    if (ptr) ptr[u] = n;
    for (int s : lists[u]) {
      if (idx) idx[n] = s;
      n++;
    }
  }
  if (ptr) ptr[ni * nj] = n;
  return n;
}

// --- FVM operator -------------------------------------------------------------
// Exports A, Gi, Gj as CSR (ascending columns).  Call once with NULL arrays to
// get the nnz counts in nnz[3].
void orc_assemble(int ni, int nj, const double* x0, const double* dh, int domain,
                  const int8_t* node_type, const int8_t* face_type, int* nnz,
                  int* a_ptr, int* a_col, double* a_val, int* gi_ptr, int* gi_col, double* gi_val,
                  int* gj_ptr, int* gj_col, double* gj_val, uint8_t* fixed) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  Operator op;
  assemble(m, op);
  std::vector<Row>* mats[3] = {&op.A, &op.Gi, &op.Gj};
  int* ptrs[3] = {a_ptr, gi_ptr, gj_ptr};
  int* cols[3] = {a_col, gi_col, gj_col};
  double* vals[3] = {a_val, gi_val, gj_val};
  for (int k = 0; k < 3; k++) {
    int n = 0;
    for (int u = 0; u < ni * nj; u++) {
      if (ptrs[k]) ptrs[k][u] = n;
      for (auto& kv : (*mats[k])[u]) {
        if (cols[k]) { cols[k][n] = kv.first; vals[k][n] = kv.second; }
        n++;
      }
    }
    if (ptrs[k]) ptrs[k][ni * nj] = n;
    nnz[k] = n;
  }
  if (fixed) memcpy(fixed, op.fixed.data(), op.fixed.size());
}

// --- nonlinear Poisson with Boltzmann electrons --------------------------------
// PoissonSolver.update + solvePotentialNL + Solver.solveNonLinearNR with the serial
// GS linear solver (PoissonSolver.java:110-252; Solver.java:293-387).
// phi: in = initial guess (previous potential), out = solution.
// bc_value: Dirichlet values.  Returns the number of NR iterations; out[0] = final
// ||y||_2, out[1] = total GS iterations.
int orc_poisson_nl(int ni, int nj, const double* x0, const double* dh, int domain,
                   const int8_t* node_type, const int8_t* face_type, const double* bc_value,
                   const double* rho, double n0, double kTe0, double phi0, double eps,
                   int max_it, double tol, int nl_max_it, double nl_tol, double* phi,
                   double* out) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  Operator op;
  assemble(m, op);
  int nu = ni * nj;
  std::vector<double> x(phi, phi + nu), b(nu);
  for (int u = 0; u < nu; u++) b[u] = rho[u] * (-1 / eps);
  for (int i = 0; i < ni; i++)
    for (int j = 0; j < nj; j++) {
      int u = j * ni + i;
      if (m.dirichlet(i, j)) { b[u] = bc_value[u]; continue; }
      if (m.nt(i, j) == NODE_INSULATOR) { b[u] = 0; continue; }
      if (i != 0 && i != ni - 1 && j != 0 && j != nj - 1) continue;
      if (i == 0 && m.bt(F_LEFT, j) != DB_MESH) b[u] = bc_value[u];
      if (i == ni - 1 && m.bt(F_RIGHT, j) != DB_MESH) b[u] = bc_value[u];
      if (j == 0 && m.bt(F_BOTTOM, i) != DB_MESH) b[u] = bc_value[u];
      if (j == ni - 1 && m.bt(F_TOP, i) != DB_MESH)  // 'ni' as written in the reference
        b[(nj - 1) * ni + i] = bc_value[(nj - 1) * ni + i];
    }
  const double C = QE / eps;
  std::vector<double> y(nu, 0.0), F(nu), bb(nu), P(nu);
  int it;
  double norm = -1;
  long total_gs = 0;
  for (it = 0; it < nl_max_it; it++) {
    for (int u = 0; u < nu; u++) {
      double ex = op.fixed[u] ? 0 : C * n0 * std::exp((x[u] - phi0) / kTe0);
      bb[u] = b[u] + ex;
      P[u] = op.fixed[u] ? 0 : C * n0 * std::exp((x[u] - phi0) / kTe0) / kTe0;
    }
    for (int i = 0; i < ni; i++)
      for (int j = 0; j < nj; j++) {
        int n = j * ni + i;
        if (m.dirichlet(i, j)) continue;
        if ((i == 0 && m.bt(F_LEFT, j) != DB_MESH && m.bt(F_LEFT, j) != DB_DIRICHLET) ||
            (i == ni - 1 && m.bt(F_RIGHT, j) != DB_MESH && m.bt(F_RIGHT, j) != DB_DIRICHLET) ||
            (j == 0 && m.bt(F_BOTTOM, i) != DB_MESH && m.bt(F_BOTTOM, i) != DB_DIRICHLET) ||
            (j == nj - 1 && m.bt(F_TOP, i) != DB_MESH && m.bt(F_TOP, i) != DB_DIRICHLET)) {
          bb[n] = 0;
          P[n] = 0;
        }
      }
    for (int u = 0; u < nu; u++) F[u] = row_mult(op.A[u], x.data()) - bb[u];
    std::vector<Row> J = op.A;
    for (int u = 0; u < nu; u++) J[u][u] -= P[u];  // Matrix.subtractDiag
    total_gs += gs_solve(J, y.data(), F.data(), nu, max_it, tol, nullptr);
    for (int u = 0; u < nu; u++) x[u] -= y[u];
    double s = 0;
    for (int u = 0; u < nu; u++) s += y[u] * y[u];
    norm = std::sqrt(s);
    if (norm < nl_tol) break;
  }
  memcpy(phi, x.data(), nu * sizeof(double));
  if (out) { out[0] = norm; out[1] = (double)total_gs; }
  return it;
}

// Nonlinear residual R = A phi - b0 - C n0 exp((phi-phi0)/kTe) on non-fixed rows,
// the quantity whose ||R||_2/N defines convergence.  Returns ||R||_2; r may be NULL.
double orc_poisson_residual(int ni, int nj, const double* x0, const double* dh, int domain,
                            const int8_t* node_type, const int8_t* face_type,
                            const double* bc_value, const double* rho, double n0, double kTe0,
                            double phi0, double eps, const double* phi, double* r) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  Operator op;
  assemble(m, op);
  int nu = ni * nj;
  const double C = QE / eps;
  double s = 0;
  for (int i = 0; i < ni; i++)
    for (int j = 0; j < nj; j++) {
      int u = j * ni + i;
      double b;
      if (op.fixed[u]) {
        b = bc_value[u];
      } else if ((i == 0 && m.bt(F_LEFT, j) != DB_MESH) || (i == ni - 1 && m.bt(F_RIGHT, j) != DB_MESH) ||
                 (j == 0 && m.bt(F_BOTTOM, i) != DB_MESH) || (j == nj - 1 && m.bt(F_TOP, i) != DB_MESH)) {
        b = 0;  // Neumann rows (the NR loop zeroes b and P there)
      } else {
        b = -rho[u] / eps + C * n0 * std::exp((phi[u] - phi0) / kTe0);
      }
      double rr = row_mult(op.A[u], phi) - b;
      if (r) r[u] = rr;
      s += rr * rr;
    }
  (void)nu;
  return std::sqrt(s);
}

// PotentialSolver.updateGradientField -> Solver.evaluateGradient with scale -1
// (PotentialSolver.java:56-70; Solver.java:789-814)
void orc_efield(int ni, int nj, const double* x0, const double* dh, int domain,
                const int8_t* node_type, const int8_t* face_type, const double* phi, double* efi,
                double* efj) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  Operator op;
  assemble(m, op);
  for (int u = 0; u < ni * nj; u++) {
    efi[u] = -row_mult(op.Gi[u], phi);
    efj[u] = -row_mult(op.Gj[u], phi);
  }
}

// BoltzmannElectronsMaterial.electronModelBoltzmann (BoltzmannElectronsMaterial.java:179-215)
void orc_boltzmann(int n, const double* phi, double n0, double kTe0, double phi0, double* den) {
  for (int u = 0; u < n; u++) {
    den[u] = n0 * std::exp((phi[u] - phi0) / kTe0);
    if (den[u] < 1) den[u] = 1;
  }
}

// --- particle push -------------------------------------------------------------
// parts: n x 12 doubles (pos[3], vel[3], lc[2], dt, mpw, alive, spare).
// segs: nseg x 9 doubles (x1, y1, x2, y2, btype, model, vth, c_rest, c_accom).
// stats out: N_sum, P_sum[3], E_sum (per-particle weights, not yet x mass),
// boundary charge.  flux/deposit: 2*nseg each (accumulated).
// rng_seed: java.util.Random seed for surface models.  threads > 1 runs the particle
// loop with OpenMP (the reference's ParticleMover threads); RNG-free surface models only.
int orc_push(int ni, int nj, const double* x0, const double* dh, int domain,
             const int8_t* node_type, const int8_t* face_type, const double* efi,
             const double* efj, double q, double mass, double dt, int nseg, const double* segs,
             const int* node_seg_ptr, const int* node_seg_idx, int n, double* parts,
             double* stats, double* flux, double* deposit, int64_t rng_seed, int threads) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  std::vector<Seg> S(nseg);
  for (int s = 0; s < nseg; s++) {
    const double* d = segs + 9 * s;
    S[s].x1[0] = d[0]; S[s].x1[1] = d[1]; S[s].x2[0] = d[2]; S[s].x2[1] = d[3];
    S[s].btype = (int)d[4]; S[s].model = (int)d[5]; S[s].vth = d[6];
    S[s].c_rest = d[7]; S[s].c_accom = d[8];
    seg_init(S[s]);
  }
  JRandom rnd;
  rnd.set_seed(rng_seed);
  for (int k = 0; k < 6; k++) stats[k] = 0;
  Particle* P = reinterpret_cast<Particle*>(parts);
  int alive_count = 0;
  if (threads <= 1) {
    PushCtx c{&m, efi, efj, q / mass, mass, q, dt, S.data(), node_seg_ptr, node_seg_idx,
              flux, deposit, 0.0, &rnd};
    for (int p = 0; p < n; p++) alive_count += push_one(c, P[p], stats);
    stats[5] = c.boundary_charge;
  } else {
#ifdef _OPENMP
    double bc = 0;
#pragma omp parallel num_threads(threads) reduction(+ : alive_count, bc)
    {
      std::vector<double> fl(2 * nseg, 0.0), dp(2 * nseg, 0.0);
      double st[5] = {0, 0, 0, 0, 0};
      JRandom r2;
      r2.set_seed(rng_seed + 7919 * omp_get_thread_num());
      PushCtx c{&m, efi, efj, q / mass, mass, q, dt, S.data(), node_seg_ptr, node_seg_idx,
                fl.data(), dp.data(), 0.0, &r2};
#pragma omp for schedule(static)
      for (int p = 0; p < n; p++) alive_count += push_one(c, P[p], st);
#pragma omp critical
      {
        for (int k = 0; k < 5; k++) stats[k] += st[k];
        for (int k = 0; k < 2 * nseg; k++) { flux[k] += fl[k]; deposit[k] += dp[k]; }
      }
      bc += c.boundary_charge;
    }
    stats[5] = bc;
#else
    return -1;
#endif
  }
  return alive_count;
}

// KineticMaterial.updateFields(md) + Material.update (KineticMaterial.java:168-197,
// Material.java:618-632): nd, u, v, w from the alive particles; nd_back added last.
void orc_update_fields(int ni, int nj, const double* x0, const double* dh, int domain,
                       const int8_t* node_type, const int8_t* face_type, const double* node_volume,
                       int n, const double* parts, double nd_back, double* den, double* U,
                       double* V, double* W) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  int nu = ni * nj;
  for (int u = 0; u < nu; u++) {
    den[u] = 0;
    if (U) U[u] = 0;
    if (V) V[u] = 0;
    if (W) W[u] = 0;
  }
  const Particle* P = reinterpret_cast<const Particle*>(parts);
  for (int p = 0; p < n; p++) {
    if (P[p].alive == 0) continue;
    scatter(m, den, P[p].lc[0], P[p].lc[1], P[p].mpw);
    if (U) scatter(m, U, P[p].lc[0], P[p].lc[1], P[p].vel[0] * P[p].mpw);
    if (V) scatter(m, V, P[p].lc[0], P[p].lc[1], P[p].vel[1] * P[p].mpw);
    if (W) scatter(m, W, P[p].lc[0], P[p].lc[1], P[p].vel[2] * P[p].mpw);
  }
  for (int u = 0; u < nu; u++) {
    double d = den[u];
    if (U) U[u] = (d != 0) ? U[u] / d : 0;
    if (V) V[u] = (d != 0) ? V[u] / d : 0;
    if (W) W[u] = (d != 0) ? W[u] / d : 0;
  }
  for (int u = 0; u < nu; u++) den[u] /= node_volume[u];
  if (nd_back != 0)
    for (int u = 0; u < nu; u++) den[u] += nd_back;
}

// KineticMaterial.updateSamples (KineticMaterial.java:1570-1595): adds the scatter of
// mpw, mpw v and mpw v^2 of every live particle to the running sums, and 1 per particle
// to the cell counter at ((int) lc0, (int) lc1).  sums: 8 node fields (count, u, v, w,
// uu, vv, ww, mpc), j-major.
void orc_update_samples(int ni, int nj, const double* x0, const double* dh, int domain,
                        const int8_t* node_type, const int8_t* face_type, int n, const double* parts,
                        double* sums) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  const size_t nu = (size_t)ni * nj;
  const Particle* P = reinterpret_cast<const Particle*>(parts);
  for (int p = 0; p < n; p++) {
    if (P[p].alive == 0) continue;
    const double w = P[p].mpw;
    const double* v = P[p].vel;
    const double a = P[p].lc[0], b = P[p].lc[1];
    scatter(m, sums + 1 * nu, a, b, w * v[0]);
    scatter(m, sums + 2 * nu, a, b, w * v[1]);
    scatter(m, sums + 3 * nu, a, b, w * v[2]);
    scatter(m, sums + 4 * nu, a, b, w * v[0] * v[0]);
    scatter(m, sums + 5 * nu, a, b, w * v[1] * v[1]);
    scatter(m, sums + 6 * nu, a, b, w * v[2] * v[2]);
    scatter(m, sums + 0 * nu, a, b, w);
    sums[7 * nu + (size_t)((int)b) * ni + (int)a] += 1;
  }
}

// KineticMaterial.computeFields (KineticMaterial.java:1606-1671) from the running sums:
// out = 10 node fields nd-ave, u-ave, v-ave, w-ave, T, T1, T2, T3, p, mpc.
void orc_compute_fields(int nu, const double* sums, int num_samples, const double* node_volume, double mass,
                        double T_init, double* out) {
  const double f = mass / KB;
  for (int u = 0; u < nu; u++) {
    const double count = sums[u];
    double T = T_init, T1 = T_init, T2 = T_init, T3 = T_init;
    if (count > 0) {
      const double U = sums[1 * nu + u] / count, V = sums[2 * nu + u] / count, W = sums[3 * nu + u] / count;
      const double uu = sums[4 * nu + u] / count - U * U;
      const double vv = sums[5 * nu + u] / count - V * V;
      const double ww = sums[6 * nu + u] / count - W * W;
      T = (uu + vv + ww) * f / 3.0;
      T1 = uu * f;
      T2 = vv * f;
      T3 = ww * f;
    }
    // Field2D.mult(1/num_samples) then scaleByVol; divideByField gives 0 where count is 0
    const double nd = count * (1.0 / num_samples) / node_volume[u];
    out[0 * nu + u] = nd;
    for (int d = 0; d < 3; d++) out[(1 + d) * nu + u] = count != 0 ? sums[(1 + d) * nu + u] / count : 0.0;
    out[4 * nu + u] = T;
    out[5 * nu + u] = T1;
    out[6 * nu + u] = T2;
    out[7 * nu + u] = T3;
    out[8 * nu + u] = nd * KB * T;
    out[9 * nu + u] = sums[7 * nu + u] * (1.0 / num_samples);
  }
}

// KineticMaterial.addParticle(md, part) (KineticMaterial.java:776-802) for XY/B=0:
// lc from pos, clamp to the mesh, rewind the velocity by -dt/2 with E at lc.
void orc_add_particles(int ni, int nj, const double* x0, const double* dh, int domain,
                       const int8_t* node_type, const int8_t* face_type, const double* efi,
                       const double* efj, double q, double mass, double dt, int n, double* parts) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  Particle* P = reinterpret_cast<Particle*>(parts);
  for (int p = 0; p < n; p++) {
    m.XtoL(P[p].pos, P[p].lc);
    if (P[p].lc[0] >= ni) P[p].lc[0] = ni - 1;
    if (P[p].lc[1] >= nj) P[p].lc[1] = nj - 1;
    P[p].dt = -0.5 * dt;
    double ef0 = gather(m, efi, P[p].lc), ef1 = gather(m, efj, P[p].lc);
    P[p].vel[0] += (q / mass) * ef0 * P[p].dt;
    P[p].vel[1] += (q / mass) * ef1 * P[p].dt;
    P[p].dt = 0;
    P[p].alive = 1;
  }
}

// MaxwellianSource.sampleParticle + Source.regenerate/sampleKinetic for a straight inlet
// segment (MaxwellianSource.java:93-125; Source.java:123-198).  Writes up to cap particles
// (pos, vel, mpw; lc/dt unset: call orc_add_particles next).  rem: in/out remainder.
// Spline.randomT on an axisymmetric mesh (core/boundaries/Spline.java:582-641): t such
// that the frustum area of [0, t] is the fraction f of the segment's; the root of
// t (2 r1 + t (r2 - r1)) / (r1 + r2) = f (the reference finds it by secant steps).
static double frustum_t(double f, double r1, double r2) {
  const double S = r1 + r2;
  if (!(S > 0.0) || f <= 0.0) return f;
  return f * S / (r1 + std::sqrt(r1 * r1 + (r2 - r1) * f * S));
}

int orc_maxwellian_source(int64_t seed, int domain, const double* seg_xy, double den, double v_drift,
                          double temp, double mass, double spwt, double dt, double* rem, int cap,
                          double* parts) {
  JRandom r;
  r.set_seed(seed);
  double x1[2] = {seg_xy[0], seg_xy[1]}, x2[2] = {seg_xy[2], seg_xy[3]};
  Seg s;
  s.x1[0] = x1[0]; s.x1[1] = x1[1]; s.x2[0] = x2[0]; s.x2[1] = x2[1];
  seg_init(s);
  double len = std::sqrt((x2[0] - x1[0]) * (x2[0] - x1[0]) + (x2[1] - x1[1]) * (x2[1] - x1[1]));
  double v_mean = std::sqrt(8 * KB * temp / (PI * mass));
  // LinearSegment.area (LinearSegment.java:51-76): length x 1 m in XY, the lateral area
  // pi (r1 + r2) L of the swept frustum in RZ / ZR
  const double r1 = domain == DOM_RZ ? x1[0] : x1[1], r2 = domain == DOM_RZ ? x2[0] : x2[1];
  double A = domain == DOM_XY ? len : PI * (r1 + r2) * len;
  double mdot = den * A * (v_drift + v_mean / 4) * mass;
  double v_th = std::sqrt(2 * KB * temp / mass);
  double mp = (mdot * dt) / (mass * spwt) + *rem;
  int num = (int)mp;
  *rem = mp - num;
  int out = 0;
  Particle* P = reinterpret_cast<Particle*>(parts);
  for (int k = 0; k < num && out < cap; k++) {
    double t = r.nextDouble();  // Boundary.randomT for a single linear segment
    if (domain != DOM_XY) t = frustum_t(t, r1, r2);
    Particle& p = P[out];
    memset(&p, 0, sizeof(Particle));
    p.pos[0] = x1[0] + t * (x2[0] - x1[0]);
    p.pos[1] = x1[1] + t * (x2[1] - x1[1]);
    const double* n = s.normal;
    do {
      double vm[3];
      sample_maxw_3d(r, v_th, vm);
      p.vel[0] = vm[0] + n[0] * v_drift;
      p.vel[1] = vm[1] + n[1] * v_drift;
      p.vel[2] = vm[2];
      p.dt = r.nextDouble() * dt;
    } while (n[0] * p.vel[0] + n[1] * p.vel[1] <= 0);
    for (int i = 0; i < 3; i++) p.pos[i] += p.vel[i] * 1e-6 * dt;
    p.mpw = spwt;
    p.alive = 1;
    out++;
  }
  return out;
}

// UniformSource (sources/UniformSource.java:36-80): the count of Source.regenerate from
// the mass flow rate, positions by Boundary.randomT (area-weighted in RZ / ZR), velocity
// normal * v_drift, then Source.sampleKinetic's 1e-6 dt push off.
int orc_uniform_source(int64_t seed, int domain, const double* seg_xy, double mdot, double v_drift, double mass,
                       double spwt, double dt, double* rem, int cap, double* parts) {
  JRandom r;
  r.set_seed(seed);
  Seg s;
  s.x1[0] = seg_xy[0]; s.x1[1] = seg_xy[1]; s.x2[0] = seg_xy[2]; s.x2[1] = seg_xy[3];
  seg_init(s);
  const double r1 = domain == DOM_RZ ? seg_xy[0] : seg_xy[1], r2 = domain == DOM_RZ ? seg_xy[2] : seg_xy[3];
  double mp = (mdot * dt) / (mass * spwt) + *rem;
  int num = (int)mp;
  *rem = mp - num;
  int out = 0;
  Particle* P = reinterpret_cast<Particle*>(parts);
  for (int k = 0; k < num && out < cap; k++) {
    double t = r.nextDouble();
    if (domain != DOM_XY) t = frustum_t(t, r1, r2);
    Particle& p = P[out];
    memset(&p, 0, sizeof(Particle));
    p.pos[0] = seg_xy[0] + t * (seg_xy[2] - seg_xy[0]);
    p.pos[1] = seg_xy[1] + t * (seg_xy[3] - seg_xy[1]);
    for (int i = 0; i < 3; i++) p.vel[i] = s.normal[i] * v_drift;
    for (int i = 0; i < 3; i++) p.pos[i] += p.vel[i] * 1e-6 * dt;
    p.mpw = spwt;
    p.alive = 1;
    out++;
  }
  return out;
}

// Spline.isOnLine (core/boundaries/Spline.java:833-862), straight segment
static bool on_line(const double* g, const double xp[2]) {
  double t;
  if (g[2] != g[0]) {
    t = (xp[0] - g[0]) / (g[2] - g[0]);
    if (t < -FLT_EPS || t > 1.0 + FLT_EPS) return false;
  } else {
    t = (xp[1] - g[1]) / (g[3] - g[1]);
    if (t < -FLT_EPS || t > 1.0 + FLT_EPS) return false;
  }
  const double d1 = g[0] + t * (g[2] - g[0]) - xp[0], d2 = g[1] + t * (g[3] - g[1]) - xp[1];
  const double l2 = (g[2] - g[0]) * (g[2] - g[0]) + (g[3] - g[1]) * (g[3] - g[1]);
  return !((d1 * d1 + d2 * d2) / l2 > FLT_EPS);
}

// BoundaryModule.isInternal (core/boundaries/BoundaryModule.java:245-251) through
// Spline.visibleSegment (Spline.java:881-929) and Spline.isInternal (:806-830)
int orc_point_internal(int nseg, const double* seg_xy, const int* seg_btype, double x, double y) {
  const double xp[2] = {x, y};
  for (int s = 0; s < nseg; s++) {
    if (seg_btype[s] == BT_VIRTUAL || seg_btype[s] == BT_OPEN) continue;
    const double* g = seg_xy + 4 * s;
    if (on_line(g, xp)) return 1;
    const double xc[2] = {0.5 * (g[0] + g[2]), 0.5 * (g[1] + g[3])};
    bool blocked = false;
    for (int s2 = 0; s2 < nseg && !blocked; s2++) {
      if (s2 == s || seg_btype[s2] == BT_VIRTUAL || seg_btype[s2] == BT_OPEN) continue;
      Seg q;
      q.x1[0] = seg_xy[4 * s2]; q.x1[1] = seg_xy[4 * s2 + 1]; q.x2[0] = seg_xy[4 * s2 + 2]; q.x2[1] = seg_xy[4 * s2 + 3];
      seg_init(q);
      double t[2];
      seg_intersect(q, xp, xc, t);
      blocked = t[0] >= 0;
    }
    if (blocked) continue;
    Seg q;
    q.x1[0] = g[0]; q.x1[1] = g[1]; q.x2[0] = g[2]; q.x2[1] = g[3];
    seg_init(q);
    const double rx = x - xc[0], ry = y - xc[1];
    const double cs = (rx * q.normal[0] + ry * q.normal[1]) / std::sqrt(rx * rx + ry * ry);
    return cs <= 0 ? 1 : 0;
  }
  return 0;
}

// VolumePreloadSource + VolumeSource (sources/VolumePreloadSource.java:44-66,
// core/source/VolumeSource.java:63-170): per cell (j-major) ceil(den cellVol / spwt) - 1
// particles uniform in the cell, SampleMaxw3D at max(temp, 50 K); internal points are
// not added; 1e-6 dt push off.  Returns the particles written (at most cap).
int orc_preload(int64_t seed, int ni, int nj, const double* x0, const double* dh, int domain, int nseg,
                const double* seg_xy, const int* seg_btype, double den, double temp, double mass, double spwt,
                double dt, int cap, double* parts) {
  JRandom r;
  r.set_seed(seed);
  const double v_th = std::sqrt(2 * KB * std::max(temp, 50.0) / mass);
  Particle* P = reinterpret_cast<Particle*>(parts);
  int out = 0;
  for (int j = 0; j < nj - 1; j++)
    for (int i = 0; i < ni - 1; i++) {
      double v = dh[0] * dh[1];
      if (domain == DOM_RZ) v *= 2 * PI * (x0[0] + (i + 0.5) * dh[0]);
      if (domain == DOM_ZR) v *= 2 * PI * (x0[1] + (j + 0.5) * dh[1]);
      double num_rem = den * v;
      while (num_rem > spwt) {
        const double ip = i + r.nextDouble(), jp = j + r.nextDouble();
        double vm[3];
        sample_maxw_3d(r, v_th, vm);
        num_rem -= spwt;
        const double px = x0[0] + ip * dh[0], py = x0[1] + jp * dh[1];
        if (orc_point_internal(nseg, seg_xy, seg_btype, px, py)) continue;
        if (out >= cap) continue;
        Particle& p = P[out];
        memset(&p, 0, sizeof(Particle));
        p.pos[0] = px;
        p.pos[1] = py;
        for (int q = 0; q < 3; q++) p.vel[q] = vm[q];
        for (int q = 0; q < 3; q++) p.pos[q] += p.vel[q] * 1e-6 * dt;
        p.lc[0] = (p.pos[0] - x0[0]) / dh[0];
        p.lc[1] = (p.pos[1] - x0[1]) / dh[1];
        p.mpw = spwt;
        p.alive = 1;
        out++;
      }
    }
  return out;
}

// --- DSMC (collisions/DSMC.java:194-454; SigmaPlus.java:38-76) ---------------------
// Single species (mat1 == mat2), fixed weight.  parts: n x 12 (lc used for binning, vel
// updated in place).  cell_state: per cell (ni-1)*(nj-1) x 2 doubles {sig_cr_max, rem}.
// sigma model: Bird 4.63 with sigma0 = pi*d^2 (two equal diameters), ref_temp, omega.
// counts: per cell {collisions, sum of weights} accumulated.
long orc_dsmc(int ni, int nj, const double* cell_vol, int n, double* parts, double mass,
              double spwt, double d_ref, double T_ref, double omega, double vss_alpha,
              double delta_t, double* cell_state, double* counts, int64_t seed) {
  JRandom rnd;
  rnd.set_seed(seed);
  int nc = (ni - 1) * (nj - 1);
  std::vector<std::vector<int>> cells(nc);
  Particle* P = reinterpret_cast<Particle*>(parts);
  // cells indexed [i][j] in the reference; the loop is i-outer, j-inner
  for (int p = 0; p < n; p++) {
    if (P[p].alive == 0) continue;
    int i = (int)P[p].lc[0], j = (int)P[p].lc[1];
    if (i >= ni - 1 || j >= nj - 1) continue;
    cells[j * (ni - 1) + i].push_back(p);
  }
  double dsum = d_ref + d_ref;
  double sigma0 = 0.25 * PI * dsum * dsum;
  double mr = mass * mass / (mass + mass);
  double gam = bird_gamma(2.5 - omega);
  double vss_inv = 0.5 * (1.0 / vss_alpha + 1.0 / vss_alpha);
  long total = 0;
  for (int i = 0; i < ni - 1; i++)
    for (int j = 0; j < nj - 1; j++) {
      int c = j * (ni - 1) + i;
      auto& L = cells[c];
      double* st = cell_state + 2 * c;
      double np1 = (double)L.size(), np2 = np1;
      double Pab = 1, Pba = 1;  // equal weights
      double nsel_f = ((np1 * spwt / cell_vol[c]) * np2 * delta_t * st[0]) / (Pab + 1.0 * Pba);
      nsel_f += st[1];
      int nsel = (int)nsel_f;
      if (np1 < 2 || np2 < 2) continue;
      st[1] = nsel_f - nsel;
      if (nsel > np1 * np2) { nsel = (int)(np1 * np2); st[1] = 0; }
      double sig_cr_max = 0;
      for (int k = 0; k < nsel; k++) {
        int p1 = (int)(rnd.nextDouble() * np1), p2;
        do { p2 = (int)(rnd.nextDouble() * np2); } while (p1 == p2);
        Particle& a = P[L[p1]];
        Particle& b = P[L[p2]];
        double cr[3] = {a.vel[0] - b.vel[0], a.vel[1] - b.vel[1], a.vel[2] - b.vel[2]};
        double cr_mag = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        double sigma = sigma0 * std::pow(2. * KB * T_ref / (mr * cr_mag * cr_mag), omega - 0.5) / gam;
        double sigma_cr = cr_mag * sigma;
        if (sigma_cr > sig_cr_max) sig_cr_max = sigma_cr;
        double Pc = sigma_cr / st[0];
        if (rnd.nextDouble() < Pc) {
          // ModelElastic.perform (DSMC.java:373-453)
          double rm1 = 0.5, rm2 = 0.5;
          double g_mag = cr_mag;
          double vc[3], vr[3];
          for (int q = 0; q < 3; q++) vc[q] = rm1 * a.vel[q] + rm2 * b.vel[q];
          if (std::fabs(vss_inv - 1.) < 1.e-4) {
            double B = 2. * rnd.nextDouble() - 1.0;
            double A = std::sqrt(1. - B * B);
            vr[0] = B * g_mag;
            double C = 2. * PI * rnd.nextDouble();
            vr[1] = A * std::cos(C) * g_mag;
            vr[2] = A * std::sin(C) * g_mag;
          } else {
            double B = 2. * (std::pow(rnd.nextDouble(), vss_inv)) - 1.;
            double A = std::sqrt(1. - B * B);
            double C = 2. * PI * rnd.nextDouble();
            double OC = std::cos(C), SC = std::sin(C);
            double D = std::sqrt(cr[1] * cr[1] + cr[2] * cr[2]);
            if (D > 1.e-6) {
              vr[0] = B * cr[0] + A * SC * D;
              vr[1] = B * cr[1] + A * (g_mag * cr[2] * OC - cr[0] * cr[1] * SC) / D;
              vr[2] = B * cr[2] - A * (g_mag * cr[1] * OC + cr[0] * cr[2] * SC) / D;
            } else {
              vr[0] = B * cr[1];
              vr[1] = A * OC * cr[1];
              vr[2] = A * SC * cr[1];
            }
          }
          for (int q = 0; q < 3; q++) {
            a.vel[q] = vc[q] + vr[q] * rm2;
            b.vel[q] = vc[q] - vr[q] * rm1;
          }
          counts[2 * c] += 1.0;
          counts[2 * c + 1] += 0.5 * (a.mpw + b.mpw);
          total++;
        }
      }
      if (sig_cr_max > 0) st[0] = sig_cr_max;
    }
  return total;
}

// DSMC.collideCell for two different kinetic materials (DSMC.java:259-350 with
// mat1 != mat2) and ModelElastic.perform with Boyd's variable-weight update
// (:373-453); SigmaBird463.init for the pair (SigmaPlus.java:54-66).  Particles of each
// species are binned by cell in array order, as the reference's iterators list them.
long orc_dsmc_pair(int ni, int nj, const double* cell_vol, int n1, double* parts1, double mass1, double spwt1,
                   int n2, double* parts2, double mass2, double spwt2, double d1, double d2, double T_ref1,
                   double T_ref2, double omega1, double omega2, double alpha1, double alpha2, double delta_t,
                   double* cell_state, double* counts, int64_t seed) {
  JRandom rnd;
  rnd.set_seed(seed);
  int nc = (ni - 1) * (nj - 1);
  std::vector<std::vector<int>> c1(nc), c2(nc);
  Particle* P1 = reinterpret_cast<Particle*>(parts1);
  Particle* P2 = reinterpret_cast<Particle*>(parts2);
  for (int p = 0; p < n1; p++) {
    if (P1[p].alive == 0) continue;
    int i = (int)P1[p].lc[0], j = (int)P1[p].lc[1];
    if (i >= ni - 1 || j >= nj - 1) continue;
    c1[j * (ni - 1) + i].push_back(p);
  }
  for (int p = 0; p < n2; p++) {
    if (P2[p].alive == 0) continue;
    int i = (int)P2[p].lc[0], j = (int)P2[p].lc[1];
    if (i >= ni - 1 || j >= nj - 1) continue;
    c2[j * (ni - 1) + i].push_back(p);
  }
  const double dsum = d1 + d2;
  const double sigma0 = 0.25 * PI * dsum * dsum;
  const double T_ref = 0.5 * (T_ref1 + T_ref2), omega = 0.5 * (omega1 + omega2);
  const double mr = mass1 * mass2 / (mass1 + mass2);
  const double gam = bird_gamma(2.5 - omega);
  const double vss_inv = 0.5 * (1.0 / alpha1 + 1.0 / alpha2);
  long total = 0;
  for (int i = 0; i < ni - 1; i++)
    for (int j = 0; j < nj - 1; j++) {
      int c = j * (ni - 1) + i;
      auto& L1 = c1[c];
      auto& L2 = c2[c];
      double* st = cell_state + 2 * c;
      double np1 = (double)L1.size(), np2 = (double)L2.size();
      double Pab = spwt2 / spwt1, Pba = spwt1 / spwt2;
      if (Pab > 1) Pab = 1;
      if (Pba > 1) Pba = 1;
      double nsel_f = ((np1 * spwt1 / cell_vol[c]) * np2 * delta_t * st[0]) / (Pab + (spwt2 / spwt1) * Pba);
      nsel_f *= 2.0;
      nsel_f += st[1];
      int nsel = (int)nsel_f;
      if (np1 < 1 || np2 < 1) continue;
      st[1] = nsel_f - nsel;
      if (nsel > np1 * np2) { nsel = (int)(np1 * np2); st[1] = 0; }
      double sig_cr_max = 0;
      for (int k = 0; k < nsel; k++) {
        int p1 = (int)(rnd.nextDouble() * np1);
        int p2 = (int)(rnd.nextDouble() * np2);
        Particle& a = P1[L1[p1]];
        Particle& b = P2[L2[p2]];
        double cr[3] = {a.vel[0] - b.vel[0], a.vel[1] - b.vel[1], a.vel[2] - b.vel[2]};
        double cr_mag = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        double sigma = sigma0 * std::pow(2. * KB * T_ref / (mr * cr_mag * cr_mag), omega - 0.5) / gam;
        double sigma_cr = cr_mag * sigma;
        if (sigma_cr > sig_cr_max) sig_cr_max = sigma_cr;
        if (rnd.nextDouble() < sigma_cr / st[0]) {
          double rm1 = mass1 / (mass1 + mass2), rm2 = mass2 / (mass1 + mass2);
          double g_mag = cr_mag;
          double vc[3], vr[3];
          for (int q = 0; q < 3; q++) vc[q] = rm1 * a.vel[q] + rm2 * b.vel[q];
          if (std::fabs(vss_inv - 1.) < 1.e-4) {
            double B = 2. * rnd.nextDouble() - 1.0;
            double A = std::sqrt(1. - B * B);
            vr[0] = B * g_mag;
            double C = 2. * PI * rnd.nextDouble();
            vr[1] = A * std::cos(C) * g_mag;
            vr[2] = A * std::sin(C) * g_mag;
          } else {
            double B = 2. * (std::pow(rnd.nextDouble(), vss_inv)) - 1.;
            double A = std::sqrt(1. - B * B);
            double C = 2. * PI * rnd.nextDouble();
            double OC = std::cos(C), SC = std::sin(C);
            double D = std::sqrt(cr[1] * cr[1] + cr[2] * cr[2]);
            if (D > 1.e-6) {
              vr[0] = B * cr[0] + A * SC * D;
              vr[1] = B * cr[1] + A * (g_mag * cr[2] * OC - cr[0] * cr[1] * SC) / D;
              vr[2] = B * cr[2] - A * (g_mag * cr[1] * OC + cr[0] * cr[2] * SC) / D;
            } else {
              vr[0] = B * cr[1];
              vr[1] = A * OC * cr[1];
              vr[2] = A * SC * cr[1];
            }
          }
          if (a.mpw == b.mpw) {
            for (int q = 0; q < 3; q++) {
              a.vel[q] = vc[q] + vr[q] * rm2;
              b.vel[q] = vc[q] - vr[q] * rm1;
            }
          } else {
            double pab = b.mpw / a.mpw, pba = a.mpw / b.mpw;
            if (rnd.nextDouble() < pab)
              for (int q = 0; q < 3; q++) a.vel[q] = vc[q] + rm2 * vr[q];
            if (rnd.nextDouble() < pba)
              for (int q = 0; q < 3; q++) b.vel[q] = vc[q] - rm1 * vr[q];
          }
          counts[2 * c] += 1.0;
          counts[2 * c + 1] += 0.5 * (a.mpw + b.mpw);
          total++;
        }
      }
      if (sig_cr_max > 0) st[0] = sig_cr_max;
    }
  return total;
}

// --- MCC (collisions/MCC.java:167-285): MEX (elastic) or CEX against a Maxwellian
// target described by node fields (den, u, v, w, T).  Constant cross-section sigma
// (SigmaConst, Sigma.java:121-126).  model: 0 = MEX, 1 = CEX.  Returns collisions.
// MCC.perform(mesh) (collisions/MCC.java:167-221) with the models MEX (:242-285), CEX
// (:287-297) and ionization (:304-356), in the reference's order of random draws.  The
// optional outputs are ni*nj node fields accumulated in place (S, count_sum, real_sum,
// delta_n) and the particles ionization creates (12 doubles each, velocities before the
// addParticle rewind, which needs E and is left to the caller).
long orc_mcc_ex(int ni, int nj, const double* x0, const double* dh, int domain, const int8_t* node_type,
                const int8_t* face_type, int n, double* parts, double src_mass, double tgt_mass, const double* tden,
                const double* tu, const double* tv, const double* tw, const double* tT, double sigma, double dt,
                int model, int64_t seed, double src_spwt, double e_ion, double prod_mass, double prod_spwt,
                double* S, double* count_sum, double* real_sum, double* delta_n, long max_new, double* new_e,
                long* n_new_e, double* new_i, long* n_new_i) {
  Mesh m = make_mesh(ni, nj, x0, dh, domain, node_type, face_type);
  JRandom rnd;
  rnd.set_seed(seed);
  Particle* P = reinterpret_cast<Particle*>(parts);
  Particle* NE = reinterpret_cast<Particle*>(new_e);
  Particle* NI = reinterpret_cast<Particle*>(new_i);
  long cols = 0, ne = 0, nion = 0;
  for (int p = 0; p < n; p++) {
    Particle& a = P[p];
    if (a.alive == 0) continue;
    double den_a = gather(m, tden, a.lc);
    if (den_a <= 0) continue;
    double tvel[3] = {gather(m, tu, a.lc), gather(m, tv, a.lc), gather(m, tw, a.lc)};
    double g_vec[3];
    for (int i = 0; i < 3; i++) g_vec[i] = tvel[i] - a.vel[i];
    double g = std::sqrt(g_vec[0] * g_vec[0] + g_vec[1] * g_vec[1] + g_vec[2] * g_vec[2]);
    double Pc = 1 - std::exp(-sigma * g * dt * den_a);
    if (Pc < rnd.nextDouble()) continue;
    // Material.sampleMaxwellianVelocity (Material.java:880-896)
    double vt[3] = {gather(m, tu, a.lc), gather(m, tv, a.lc), gather(m, tw, a.lc)};
    double T = gather(m, tT, a.lc);
    if (T < 0) T = 0;
    double v_th = std::sqrt(2 * KB * T / tgt_mass);
    double vm[3];
    sample_maxw_3d(rnd, v_th, vm);
    for (int i = 0; i < 3; i++) vt[i] += vm[i];
    const double E1 = 0.5 * src_mass * std::sqrt(a.vel[0] * a.vel[0] + a.vel[1] * a.vel[1] + a.vel[2] * a.vel[2]);
    if (model == 2) {
      double e1 = 0.5 * src_mass * (a.vel[0] * a.vel[0] + a.vel[1] * a.vel[1] + a.vel[2] * a.vel[2]) / QE;
      double e2 = e1 - e_ion;
      if (e2 >= 0) {
        double e2a = rnd.nextDouble() * e2;
        double speed2a = std::sqrt(e2a * QE * 2 / src_mass);
        isotropic_vel(rnd, speed2a, a.vel);
        double Tt = gather(m, tT, a.lc);  // getTempCollection().eval(pos, 300) inside the mesh
        if (Tt <= 0) Tt = 100;
        double v2b[3];
        isotropic_vel(rnd, speed2a, v2b);  // the reference's speed2a, not speed2b
        if (NE && ne < max_new) {
          Particle q = a;
          for (int i = 0; i < 3; i++) q.vel[i] = v2b[i];
          NE[ne] = q;
        }
        ne++;
        int mp_gen = (int)(src_spwt / prod_spwt + rnd.nextDouble());
        if (mp_gen > 0) {
          double vth_i = std::sqrt(2 * KB * Tt / prod_mass);
          for (int k = 0; k < mp_gen; k++) {
            double v3[3];
            sample_maxw_3d(rnd, vth_i, v3);
            if (NI && nion < max_new) {
              Particle q = a;
              for (int i = 0; i < 3; i++) q.vel[i] = v3[i];
              q.mpw = prod_spwt;
              NI[nion] = q;
            }
            nion++;
          }
          if (delta_n) delta_n[(int)a.lc[1] * ni + (int)a.lc[0]] += prod_spwt * mp_gen;
        }
      }
    } else if (model == 1) {
      for (int i = 0; i < 3; i++) a.vel[i] = vt[i];
    } else {
      double rm1 = src_mass / (src_mass + tgt_mass), rm2 = tgt_mass / (src_mass + tgt_mass);
      double gg[3], vc[3], vr[3];
      for (int i = 0; i < 3; i++) gg[i] = a.vel[i] - vt[i];
      double g_mag = std::sqrt(gg[0] * gg[0] + gg[1] * gg[1] + gg[2] * gg[2]);
      for (int i = 0; i < 3; i++) vc[i] = rm1 * a.vel[i] + rm2 * vt[i];
      double B = 2. * rnd.nextDouble() - 1.0;
      double A = std::sqrt(1. - B * B);
      vr[0] = B * g_mag;
      double C = 2. * PI * rnd.nextDouble();
      vr[1] = A * std::cos(C) * g_mag;
      vr[2] = A * std::sin(C) * g_mag;
      for (int i = 0; i < 3; i++) a.vel[i] = vc[i] + vr[i] * rm2;
    }
    // target energy term and collision counts (MCC.java:204-218)
    const double E2 = 0.5 * src_mass * std::sqrt(a.vel[0] * a.vel[0] + a.vel[1] * a.vel[1] + a.vel[2] * a.vel[2]);
    if (S) scatter(m, S, a.lc[0], a.lc[1], a.mpw * (E1 - E2) / (dt * node_vol(m, a.lc[0], a.lc[1])));
    const int u = (int)a.lc[1] * ni + (int)a.lc[0];
    if (count_sum) count_sum[u] += 1;
    if (real_sum) real_sum[u] += a.mpw;
    cols++;
  }
  if (n_new_e) *n_new_e = ne;
  if (n_new_i) *n_new_i = nion;
  return cols;
}

long orc_mcc(int ni, int nj, const double* x0, const double* dh, int domain, const int8_t* node_type,
             const int8_t* face_type, int n, double* parts, double src_mass, double tgt_mass, const double* tden,
             const double* tu, const double* tv, const double* tw, const double* tT, double sigma, double dt,
             int model, int64_t seed) {
  return orc_mcc_ex(ni, nj, x0, dh, domain, node_type, face_type, n, parts, src_mass, tgt_mass, tden, tu, tv, tw, tT,
                    sigma, dt, model, seed, 1.0, 0.0, 1.0, 1.0, nullptr, nullptr, nullptr, nullptr, 0, nullptr,
                    nullptr, nullptr, nullptr);
}

}  // extern "C"
