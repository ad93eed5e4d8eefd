// Dipole-dipole field by FFT convolution (the "dipole-fft" Hamiltonian,
// src/jams/hamiltonian/cuda_dipole_fft.cu:19-343).  Host interface.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "llg_internal.h"

namespace jams_llg {

struct DipoleGeometry {
  double r_cutoff;            // lattice parameters
  double tolerance;           // lattice parameters
  double a;                   // lattice parameter (m)
  double A[9];                // lattice vectors a1, a2, a3 (rows, lattice parameters)
  double frac[kMaxBasis][3];  // fractional basis positions
};

struct DipoleReplicaSpec {
  int L[3];
  int64_t offset;             // first spin of the replica in every state plane
};

struct DipoleField;

// Builds the k-space tensors, transform plans and twiddle tables of every
// replica.  Returns null and sets err when the geometry is invalid (cutoff
// beyond the inradius of the periodic supercell, coincident sites, a grid
// axis longer than one shared-memory transform line of the FP64 tensor
// transforms, 4842 points) or a CUDA call fails.
DipoleField* dipole_create(const DipoleGeometry& g, int nb, const int periodic[3], const double* mus,
                           const std::vector<DipoleReplicaSpec>& reps, bool fp64, std::string& err);
void dipole_destroy(DipoleField* d);
// kernel launches of one field evaluation, over all replicas: per replica
// the forward real pass, one complex pass per further grid axis longer than
// one cell, the k-space product, the complex passes back and the inverse
// real pass
int64_t dipole_launches(const DipoleField* d);

// Dipole field (meV) of the state planes `s` (three planes of npad reals,
// float or double as at creation) into `h` (same layout), on stream st.
// Returns a message on failure, empty on success.
std::string dipole_compute(DipoleField* d, const void* s, void* h, int64_t npad, cudaStream_t st);

// bytes of device memory held (tensors, grids, FFT work areas)
size_t dipole_device_bytes(const DipoleField* d);

// the largest cutoff the periodic supercell allows (lattice parameters):
// jams::maximum_interaction_length, src/jams/core/lattice.cc:1155-1200
double dipole_max_radius(const double A[9], const int L[3], const int periodic[3]);

}  // namespace jams_llg
