// frame.h -- arbitrary-axis cylinders (AXX_PRIM_CYLINDER) by a change of frame.
//
// The reference's Cylinder (src/primitives/cylinder.cuh:1-199, a draft that
// does not compile) is an infinite cylinder through a centre along any axis,
// described in the frame (ahat, bhat, chat) it builds from the axis: chat =
// axis, ahat = chat x z (x when the axis is along z), bhat = chat x ahat.  In
// that frame it is a Cylinder_XY.  The walk is the same physics in any
// orthonormal frame: positions r_f = R r, gradient directions g_f = R g (so
// the phase G . r is unchanged), while cell sides and the other bases follow.
// So instead of a second kernel geometry, the host rewrites the substrate and
// the sequences into the frame where every cylinder runs along z, and traces
// are rotated back (exactly, for the permutation frames of lattices).
//
//   * single pores: R has the rows (ahat, bhat, chat) of the reference's
//     construction; the pore becomes a Cylinder_XY at (ahat.c, bhat.c);
//   * lattices: the cell is axis-aligned, so a periodic lattice of cylinders
//     needs their common axis along a cell axis; R is the cyclic permutation
//     that takes that axis to z (x -> (y, z, x), y -> (z, x, y)).
#pragma once

#include <string>
#include <vector>

#include "../../include/axx.h"

namespace axx {

struct Frame {
  bool identity = true;
  double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};  // r_frame = R r
  axx_lattice lat{};
  std::vector<axx_basis> basis;
  std::vector<axx_sequence> seqs;
  // inputs to use: the originals when identity, else the rewritten copies
  const axx_lattice *lat_p = nullptr;
  const axx_basis *basis_p = nullptr;
  const axx_sequence *seqs_p = nullptr;
};

// Returns "" on success or an error message.  seqs may be null (nseq 0).
std::string frame_lattice(const axx_lattice *lat, const axx_basis *basis, int nbasis,
                          const axx_sequence *seqs, int nseq, Frame &f);
std::string frame_single(const axx_basis *pore, const axx_sequence *seqs, int nseq, Frame &f);

// Rotates n points (x, y, z float triples) from the frame back to the
// simulation coordinates: r = R^T r_frame.
void frame_to_sim(const Frame &f, float *xyz, size_t n);
// The same for a 3x3 rotation held elsewhere (plans keep R).
void frame_to_sim(const double R[3][3], float *xyz, size_t n);

}  // namespace axx
