// Output pipeline: recompute_at_gausspts_beams! and recompute_at_nodes_beams!
// (src/IO/visualization_beams.jl:122-175) as device kernels, and an
// asynchronous VTK PolyData writer (write_VTK_beams, :74-120) that formats and
// writes the files on its own host thread while the batch keeps stepping.
#pragma once
#include <string>
#include <vector>

#include "eb_internal.cuh"

namespace eb {

// Per-simulation output block, NP = n_elem * pts points:
//   [x (3 NP) | displacement (3 NP) | velocity (3 NP) | strain (NP) | stress (NP)]
// The writer's staging slots append [x (3 n) | displacement (3 n)] of the n nodes.
inline int64_t beam_output_doubles(int64_t n_elem, int pts) { return 11 * n_elem * (int64_t)pts; }
inline int64_t node_output_doubles(int64_t n_nodes) { return 6 * n_nodes; }

// Elements [e0, e0 + ne) and nodes [n0, n0 + nn) of one simulation, current state (u, u̇, R).
void launch_beam_output(const Dev& d, const double* E, int64_t e0, int64_t ne, int pts, double* out, cudaStream_t s);
void launch_node_output(const Dev& d, int64_t n0, int64_t nn, double* out, cudaStream_t s);

struct VtkWriter;

struct VtkSim {
  int64_t e0, ne, n0, nn;  // element / node ranges of the simulation in the batch
};

// Opens the writer: one output directory per simulation ("" = none), created if missing.
// Returns nullptr and sets `err` on failure.
VtkWriter* vtk_open(const Dev& d, const double* E, cudaStream_t stream, const std::vector<VtkSim>& sims,
                    const std::vector<std::string>& dirs, int pts, std::string& err);
// Queues the files of the simulations in `mask` (state of the handle's stream at this point).
int vtk_write(VtkWriter* w, const int32_t* mask, const int32_t* counter, const int32_t* step, const double* t,
              std::string& err);
// Waits until every queued file is written; returns nonzero with `err` set if a write failed.
int vtk_flush(VtkWriter* w, std::string& err);
// Flushes, writes each directory's simulation.pvd and frees the writer.
int vtk_close(VtkWriter* w, std::string& err);

}  // namespace eb
