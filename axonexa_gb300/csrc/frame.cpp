// frame.cpp -- the change of frame that turns arbitrary-axis cylinders into
// cylinders along z (see frame.h).
#include "frame.h"

#include <cmath>

namespace axx {
namespace {

bool finite3(double x, double y, double z) {
  return std::isfinite(x) && std::isfinite(y) && std::isfinite(z);
}

// Unit axis of an AXX_PRIM_CYLINDER, or false.
bool unit_axis(const axx_basis &b, double a[3]) {
  if (!finite3(b.nx, b.ny, b.nz)) return false;
  const double m = std::sqrt(b.nx * b.nx + b.ny * b.ny + b.nz * b.nz);
  if (!(m > 1e-12)) return false;
  a[0] = b.nx / m;
  a[1] = b.ny / m;
  a[2] = b.nz / m;
  return true;
}

void apply(const double R[3][3], double x, double y, double z, double out[3]) {
  for (int i = 0; i < 3; ++i) out[i] = R[i][0] * x + R[i][1] * y + R[i][2] * z;
}

void rotate_seqs(Frame &f, const axx_sequence *seqs, int nseq) {
  f.seqs.assign(seqs, seqs + nseq);
  for (auto &q : f.seqs) {
    double g[3];
    apply(f.R, q.gx, q.gy, q.gz, g);
    q.gx = g[0];
    q.gy = g[1];
    q.gz = g[2];
  }
}

void use_originals(Frame &f, const axx_lattice *lat, const axx_basis *basis,
                   const axx_sequence *seqs) {
  f.identity = true;
  f.lat_p = lat;
  f.basis_p = basis;
  f.seqs_p = seqs;
}

}  // namespace

std::string frame_single(const axx_basis *pore, const axx_sequence *seqs, int nseq, Frame &f) {
  f = Frame();
  if (!pore || pore->type != AXX_PRIM_CYLINDER) {
    use_originals(f, nullptr, pore, seqs);
    return "";
  }
  double c[3];
  if (!unit_axis(*pore, c)) return "cylinder axis must be finite and nonzero";
  // cylinder.cuh:20-40: chat = axis, ahat = chat x z (x, y when the axis is
  // along z), bhat = chat x ahat, both normalised
  double a[3] = {c[1], -c[0], 0.0}, b[3];
  const double am = std::sqrt(a[0] * a[0] + a[1] * a[1]);
  if (am < 1e-14) {
    a[0] = 1.0;
    a[1] = 0.0;
    b[0] = 0.0;
    b[1] = 1.0;
    b[2] = 0.0;
  } else {
    a[0] /= am;
    a[1] /= am;
    b[0] = c[1] * a[2] - c[2] * a[1];
    b[1] = c[2] * a[0] - c[0] * a[2];
    b[2] = c[0] * a[1] - c[1] * a[0];
    const double bm = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    for (double &v : b) v /= bm;
  }
  for (int j = 0; j < 3; ++j) {
    f.R[0][j] = a[j];
    f.R[1][j] = b[j];
    f.R[2][j] = c[j];
  }
  f.identity = false;
  axx_basis q = *pore;
  double cf[3];
  apply(f.R, pore->cx, pore->cy, pore->cz, cf);
  q.type = AXX_PRIM_CYLINDER_Z;
  q.cx = cf[0];
  q.cy = cf[1];
  q.cz = 0.0;
  q.nx = q.ny = q.nz = 0.0;
  f.basis.assign(1, q);
  rotate_seqs(f, seqs, nseq);
  f.basis_p = f.basis.data();
  f.seqs_p = f.seqs.data();
  return "";
}

std::string frame_lattice(const axx_lattice *lat, const axx_basis *basis, int nbasis,
                          const axx_sequence *seqs, int nseq, Frame &f) {
  f = Frame();
  int axis = -1;  // common cell axis of the AXX_PRIM_CYLINDER bases
  bool any_z = false;
  for (int k = 0; k < nbasis && basis; ++k) {
    if (basis[k].type == AXX_PRIM_CYLINDER_Z) any_z = true;
    if (basis[k].type != AXX_PRIM_CYLINDER) continue;
    double a[3];
    if (!unit_axis(basis[k], a)) return "cylinder axis must be finite and nonzero";
    int along = -1;
    for (int i = 0; i < 3; ++i)
      if (std::fabs(std::fabs(a[i]) - 1.0) < 1e-12) along = i;
    if (along < 0)
      return "a lattice cylinder's axis must lie along a cell axis (x, y or z): tilted "
             "cylinders do not tile an axis-aligned periodic cell";
    if (axis >= 0 && along != axis) return "the cylinders of one lattice must share an axis";
    axis = along;
  }
  if (axis < 0) {
    use_originals(f, lat, basis, seqs);
    return "";
  }
  if (any_z && axis != 2)
    return "z-axis cylinders (Cylinder_XY) and cylinders along another cell axis cannot share "
           "a lattice";
  // cyclic permutation taking the cylinders' axis to z: x -> (y, z, x),
  // y -> (z, x, y), z -> identity
  const int perm[3][3] = {{1, 2, 0}, {2, 0, 1}, {0, 1, 2}};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) f.R[i][j] = perm[axis][i] == j ? 1.0 : 0.0;
  f.identity = axis == 2;
  if (lat) {
    f.lat = *lat;
    const double side[3] = {lat->a, lat->b, lat->c};
    f.lat.a = side[perm[axis][0]];
    f.lat.b = side[perm[axis][1]];
    f.lat.c = side[perm[axis][2]];
  }
  f.basis.assign(basis, basis + nbasis);
  for (auto &q : f.basis) {
    double c[3], n[3];
    apply(f.R, q.cx, q.cy, q.cz, c);
    apply(f.R, q.nx, q.ny, q.nz, n);
    q.cx = c[0];
    q.cy = c[1];
    q.cz = c[2];
    q.nx = n[0];
    q.ny = n[1];
    q.nz = n[2];
    if (q.type == AXX_PRIM_CYLINDER) {  // as a Cylinder_XY record
      q.type = AXX_PRIM_CYLINDER_Z;
      q.cz = 0.0;
      q.nx = q.ny = q.nz = 0.0;
    }
  }
  rotate_seqs(f, seqs, nseq);
  f.lat_p = lat ? &f.lat : nullptr;
  f.basis_p = f.basis.data();
  f.seqs_p = f.seqs.data();
  return "";
}

void frame_to_sim(const double R[3][3], float *xyz, size_t n) {
  for (size_t p = 0; p < n; ++p) {
    const double x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
    for (int j = 0; j < 3; ++j)
      xyz[3 * p + j] = (float)(R[0][j] * x + R[1][j] * y + R[2][j] * z);
  }
}

void frame_to_sim(const Frame &f, float *xyz, size_t n) {
  if (!f.identity) frame_to_sim(f.R, xyz, n);
}

}  // namespace axx
