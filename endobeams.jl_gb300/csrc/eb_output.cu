// Output pipeline (see eb_output.cuh).
//
// Device side: one thread per element evaluates the element frame once and
// writes its `pts` interpolated points in the file's own array layout
// (interleaved xyz, then the scalar fields), so the host writes the staged
// block to disk as it arrives.  Host side: two staging slots (device buffer +
// pinned host buffer).  A write launches the kernels on the handle's stream,
// copies the slot to pinned memory on a separate copy stream and queues the
// file job; a writer thread waits for the copy, formats the VTK XML header
// and streams the appended raw arrays to disk.  The caller's stream only
// waits for a slot when the writer is two files behind.
#include <sys/stat.h>

#include <cerrno>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>

#include "eb_output.cuh"

namespace eb {
using namespace ebd;

namespace {

__device__ __forceinline__ V3 ld_node(const double* f, int64_t n, int64_t i) {
  return v3(f[i], f[n + i], f[2 * n + i]);
}

// recompute_at_gausspts_beams! (visualization_beams.jl:122-162), one thread per element.
__global__ void k_beam_output(Dev d, const double* __restrict__ E, int64_t e0, int64_t ne, int pts,
                              double* __restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ne) return;
  const int64_t e = e0 + j, n = d.n_nodes, NE = d.n_elem, NP = ne * pts;
  const int a = d.ea[e], b = d.eb[e];
  const V3 u1 = ld_node(d.u, n, a), u2 = ld_node(d.u, n, b);
  const V3 v1 = ld_node(d.ud, n, a), v2 = ld_node(d.ud, n, b);
  const V3 x1 = ld_node(d.X0, n, a) + u1, x2 = ld_node(d.X0, n, b) + u2;
  M3 R1, R2, Re0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    R1.a[k] = d.R[k * n + a];
    R2.a[k] = d.R[k * n + b];
    Re0.a[k] = d.Re0[k * NE + e];
  }
  const double l0 = d.l0[e];
  const double ln = norm(x2 - x1);
  const Frame f = local_frame(x1, x2, R1, R2, col(Re0, 1), ln);
  const V3 T1 = toangle(mulTN(f.Re, R1) * Re0);
  const V3 T2 = toangle(mulTN(f.Re, R2) * Re0);
  const double strain = 1 - ln / l0, stress = E[e] * (1 - ln / l0);
  double* ox = out;
  double* od = out + 3 * NP;
  double* ov = out + 6 * NP;
  double* oe = out + 9 * NP;
  double* os = out + 10 * NP;
  for (int i = 0; i < pts; ++i) {
    const int64_t k = j * pts + i;
    // z = range(-1, 1, length = pts)[i + 1], correctly rounded
    const double z = (2.0 * i - (pts - 1)) / (double)(pts - 1);
    const double xi = l0 * (z + 1) / 2;
    const double N1 = 1 - xi / l0, N2 = 1 - N1;
    const double N3 = xi * ((1 - xi / l0) * (1 - xi / l0));
    const double N4 = -(1 - xi / l0) * ((xi * xi) / l0);
    const V3 ut = v3(0.0, N3 * T1.z + N4 * T2.z, -N3 * T1.y - N4 * T2.y);
    const V3 xg = (N1 * x1 + N2 * x2) + f.Re * ut;
    const V3 dg = N1 * u1 + N2 * u2;
    const V3 vg = N1 * v1 + N2 * v2;
    ox[3 * k] = xg.x; ox[3 * k + 1] = xg.y; ox[3 * k + 2] = xg.z;
    od[3 * k] = dg.x; od[3 * k + 1] = dg.y; od[3 * k + 2] = dg.z;
    ov[3 * k] = vg.x; ov[3 * k + 1] = vg.y; ov[3 * k + 2] = vg.z;
    oe[k] = strain;
    os[k] = stress;
  }
}

// recompute_at_nodes_beams! (visualization_beams.jl:165-175): positions and displacements.
__global__ void k_node_output(Dev d, int64_t n0, int64_t nn, double* __restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nn) return;
  const int64_t i = n0 + j, n = d.n_nodes;
  const V3 u = ld_node(d.u, n, i);
  const V3 x = ld_node(d.X0, n, i) + u;
  out[3 * j] = x.x; out[3 * j + 1] = x.y; out[3 * j + 2] = x.z;
  out[3 * nn + 3 * j] = u.x; out[3 * nn + 3 * j + 1] = u.y; out[3 * nn + 3 * j + 2] = u.z;
}

}  // namespace

void launch_beam_output(const Dev& d, const double* E, int64_t e0, int64_t ne, int pts, double* out, cudaStream_t s) {
  if (ne > 0) k_beam_output<<<nblocks(ne, 128), 128, 0, s>>>(d, E, e0, ne, pts, out);
}

void launch_node_output(const Dev& d, int64_t n0, int64_t nn, double* out, cudaStream_t s) {
  if (nn > 0) k_node_output<<<nblocks(nn, 256), 256, 0, s>>>(d, n0, nn, out);
}

// ------------------------------------------------------------------ VTK writer

namespace {

struct Slot {
  double* dev = nullptr;
  double* host = nullptr;  // pinned
  cudaEvent_t ready = nullptr, copied = nullptr;
  bool busy = false, copied_recorded = false;
};

struct Job {
  int slot, sim;
  int32_t counter, step;
  double t;
};

struct PvdEntry {
  double t;
  std::string beams, nodes;
};

bool make_dirs(const std::string& path) {
  if (path.empty()) return false;
  std::string cur;
  size_t i = 0;
  while (i <= path.size()) {
    size_t j = path.find('/', i);
    if (j == std::string::npos) j = path.size();
    cur = path.substr(0, j);
    if (!cur.empty()) {
      struct stat st;
      if (stat(cur.c_str(), &st) != 0) {
        if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
      } else if (!S_ISDIR(st.st_mode)) {
        return false;
      }
    }
    i = j + 1;
  }
  return true;
}

// Appended-raw VTK XML PolyData (UInt64 block headers, little endian), the layout
// WriteVTK.jl produces for vtk_grid(filename, points, lines) without compression.
struct VtpFile {
  struct Array {
    const char* type;  // "Float64" | "Int64"
    std::string name;
    int comps;
    const void* data;  // nullptr: zeros
    uint64_t count;    // values (tuples x comps)
    const char* section;
  };
  std::vector<Array> arrays;
  int64_t n_points = 0, n_lines = 0;
  std::string error;

  void add(const char* section, const char* type, const std::string& name, int comps, const void* data,
           uint64_t count) {
    arrays.push_back(Array{type, name, comps, data, count, section});
  }

  bool write(const std::string& path) {
    FILE* fp = std::fopen(path.c_str(), "wb");
    if (!fp) {
      error = "cannot open " + path + ": " + std::strerror(errno);
      return false;
    }
    std::vector<uint64_t> offs(arrays.size());
    uint64_t off = 0;
    for (size_t k = 0; k < arrays.size(); ++k) {
      offs[k] = off;
      off += 8 + 8 * arrays[k].count;
    }
    std::string x;
    char buf[512];
    x += "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n";
    x += "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n";
    x += "  <PolyData>\n";
    auto section = [&](const char* sec, const char* indent) {
      for (size_t k = 0; k < arrays.size(); ++k) {
        const Array& a = arrays[k];
        if (std::strcmp(a.section, sec) != 0) continue;
        if (std::strcmp(sec, "FieldData") == 0)
          std::snprintf(buf, sizeof(buf),
                        "%s<DataArray type=\"%s\" Name=\"%s\" NumberOfTuples=\"%llu\" format=\"appended\" "
                        "offset=\"%llu\"/>\n",
                        indent, a.type, a.name.c_str(), (unsigned long long)a.count, (unsigned long long)offs[k]);
        else
          std::snprintf(buf, sizeof(buf),
                        "%s<DataArray type=\"%s\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"appended\" "
                        "offset=\"%llu\"/>\n",
                        indent, a.type, a.name.c_str(), a.comps, (unsigned long long)offs[k]);
        x += buf;
      }
    };
    x += "    <FieldData>\n";
    section("FieldData", "      ");
    x += "    </FieldData>\n";
    std::snprintf(buf, sizeof(buf),
                  "    <Piece NumberOfPoints=\"%lld\" NumberOfVerts=\"0\" NumberOfLines=\"%lld\" "
                  "NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n",
                  (long long)n_points, (long long)n_lines);
    x += buf;
    x += "      <Points>\n";
    section("Points", "        ");
    x += "      </Points>\n      <Lines>\n";
    section("Lines", "        ");
    x += "      </Lines>\n      <PointData>\n";
    section("PointData", "        ");
    x += "      </PointData>\n    </Piece>\n  </PolyData>\n  <AppendedData encoding=\"raw\">\n_";
    bool ok = std::fwrite(x.data(), 1, x.size(), fp) == x.size();
    static const uint64_t kZeros[512] = {0};
    for (size_t k = 0; ok && k < arrays.size(); ++k) {
      const Array& a = arrays[k];
      const uint64_t nbytes = 8 * a.count;
      ok = std::fwrite(&nbytes, 8, 1, fp) == 1;
      if (!ok) break;
      if (a.data) {
        ok = std::fwrite(a.data, 8, a.count, fp) == a.count;
      } else {
        for (uint64_t left = a.count; ok && left > 0;) {
          const uint64_t c = left < 512 ? left : 512;
          ok = std::fwrite(kZeros, 8, c, fp) == c;
          left -= c;
        }
      }
    }
    const char* tail = "\n  </AppendedData>\n</VTKFile>\n";
    ok = ok && std::fwrite(tail, 1, std::strlen(tail), fp) == std::strlen(tail);
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) error = "write failed: " + path;
    return ok;
  }
};

}  // namespace

struct VtkWriter {
  Dev d{};
  const double* E = nullptr;
  cudaStream_t stream = nullptr, copy = nullptr;
  int device = 0;
  int pts = 10;
  std::vector<VtkSim> sims;
  std::vector<std::string> dirs;
  std::vector<std::vector<int64_t>> lines;  // per simulation with output: local node pairs of its elements
  std::vector<std::vector<PvdEntry>> pvd;
  std::vector<int64_t> iota, offsets;       // beams file connectivity / offsets, sized for the largest simulation
  Slot slot[2];
  int next = 0;
  size_t slot_doubles = 0;
  // writer thread
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job> queue;
  int pending = 0;
  bool stop = false;
  std::string error;

  void run() {
    cudaSetDevice(device);
    while (true) {
      Job job;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !queue.empty(); });
        if (queue.empty()) return;
        job = queue.front();
        queue.pop_front();
      }
      std::string err = write_job(job);
      {
        std::lock_guard<std::mutex> lk(mu);
        if (!err.empty() && error.empty()) error = err;
        slot[job.slot].busy = false;
        --pending;
      }
      cv.notify_all();
    }
  }

  std::string write_job(const Job& job) {
    Slot& sl = slot[job.slot];
    cudaError_t e = cudaEventSynchronize(sl.copied);
    if (e != cudaSuccess) return std::string("output copy failed: ") + cudaGetErrorString(e);
    const VtkSim& S = sims[job.sim];
    const int64_t NP = S.ne * pts;
    const double* h = sl.host;
    const std::string& dir = dirs[job.sim];
    const std::string fb = "beams_" + std::to_string(job.counter) + ".vtp";
    const std::string fn = "beams_nodes_" + std::to_string(job.counter) + ".vtp";
    const int64_t step = job.step;
    // write_VTK_beams (visualization_beams.jl:85-101): interpolated beams
    VtpFile b;
    b.n_points = NP;
    b.n_lines = S.ne;
    b.add("FieldData", "Float64", "time", 1, &job.t, 1);
    b.add("FieldData", "Int64", "step", 1, &step, 1);
    b.add("Points", "Float64", "Points", 3, h, 3 * NP);
    b.add("Lines", "Int64", "connectivity", 1, iota.data(), NP);
    b.add("Lines", "Int64", "offsets", 1, offsets.data(), S.ne);
    b.add("PointData", "Float64", "Stress", 1, h + 10 * NP, NP);
    b.add("PointData", "Float64", "Strain", 1, h + 9 * NP, NP);
    b.add("PointData", "Float64", "Displacement", 3, h + 3 * NP, 3 * NP);
    b.add("PointData", "Float64", "Velocity", 3, h + 6 * NP, 3 * NP);
    if (!b.write(dir + "/" + fb)) return b.error;
    // nodes (visualization_beams.jl:104-117); the reference never updates the nodes'
    // contact fields (def_node_beam.jl:46-47), so they are written as zeros
    const double* hn = h + 11 * NP;
    std::vector<int64_t> node_off(S.ne);
    for (int64_t k = 0; k < S.ne; ++k) node_off[k] = 2 * (k + 1);
    VtpFile n;
    n.n_points = S.nn;
    n.n_lines = S.ne;
    n.add("FieldData", "Float64", "time", 1, &job.t, 1);
    n.add("FieldData", "Int64", "step", 1, &step, 1);
    n.add("Points", "Float64", "Points", 3, hn, 3 * S.nn);
    n.add("Lines", "Int64", "connectivity", 1, lines[job.sim].data(), 2 * S.ne);
    n.add("Lines", "Int64", "offsets", 1, node_off.data(), S.ne);
    n.add("PointData", "Float64", "Displacement", 3, hn + 3 * S.nn, 3 * S.nn);
    n.add("PointData", "Int64", "In Contact", 1, nullptr, S.nn);
    n.add("PointData", "Float64", "Contact Force", 3, nullptr, 3 * S.nn);
    n.add("PointData", "Float64", "Contact Distance", 1, nullptr, S.nn);
    if (!n.write(dir + "/" + fn)) return n.error;
    pvd[job.sim].push_back(PvdEntry{job.t, fb, fn});
    return "";
  }

  void free_all() {
    for (Slot& s : slot) {
      if (s.dev) cudaFree(s.dev);
      if (s.host) cudaFreeHost(s.host);
      if (s.ready) cudaEventDestroy(s.ready);
      if (s.copied) cudaEventDestroy(s.copied);
      s = Slot{};
    }
    if (copy) cudaStreamDestroy(copy);
    copy = nullptr;
  }
};

VtkWriter* vtk_open(const Dev& d, const double* E, cudaStream_t stream, const std::vector<VtkSim>& sims,
                    const std::vector<std::string>& dirs, int pts, std::string& err) {
  if (pts < 2) {
    err = "points_per_beam must be at least 2";
    return nullptr;
  }
  auto* w = new VtkWriter();
  w->d = d;
  w->E = E;
  w->stream = stream;
  w->pts = pts;
  w->sims = sims;
  w->dirs = dirs;
  w->lines.resize(sims.size());
  w->pvd.resize(sims.size());
  cudaGetDevice(&w->device);
  int64_t max_ne = 0;
  size_t need = 0;
  std::vector<int> ea, eb;
  for (size_t s = 0; s < sims.size(); ++s) {
    if (dirs[s].empty()) continue;
    if (!make_dirs(dirs[s])) {
      err = "cannot create output directory " + dirs[s];
      delete w;
      return nullptr;
    }
    const VtkSim& S = sims[s];
    max_ne = std::max(max_ne, S.ne);
    need = std::max(need, (size_t)(beam_output_doubles(S.ne, pts) + node_output_doubles(S.nn)));
    // local node pairs of the simulation's elements (lines of the nodes file)
    ea.resize(S.ne);
    eb.resize(S.ne);
    cudaError_t e = cudaMemcpy(ea.data(), d.ea + S.e0, sizeof(int) * S.ne, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(eb.data(), d.eb + S.e0, sizeof(int) * S.ne, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      err = std::string("vtk_open: ") + cudaGetErrorString(e);
      delete w;
      return nullptr;
    }
    auto& L = w->lines[s];
    L.resize(2 * S.ne);
    for (int64_t k = 0; k < S.ne; ++k) {
      L[2 * k] = ea[k] - S.n0;
      L[2 * k + 1] = eb[k] - S.n0;
    }
  }
  w->iota.resize(max_ne * pts);
  for (int64_t k = 0; k < max_ne * pts; ++k) w->iota[k] = k;
  w->offsets.resize(max_ne);
  for (int64_t k = 0; k < max_ne; ++k) w->offsets[k] = (k + 1) * pts;
  w->slot_doubles = need;
  if (need > 0) {
    cudaError_t e = cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking);
    for (Slot& sl : w->slot) {
      if (e == cudaSuccess) e = cudaMalloc(&sl.dev, sizeof(double) * need);
      if (e == cudaSuccess) e = cudaMallocHost(&sl.host, sizeof(double) * need);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
      err = std::string("vtk_open: ") + cudaGetErrorString(e);
      w->free_all();
      delete w;
      return nullptr;
    }
  }
  w->th = std::thread([w] { w->run(); });
  return w;
}

int vtk_write(VtkWriter* w, const int32_t* mask, const int32_t* counter, const int32_t* step, const double* t,
              std::string& err) {
  for (size_t s = 0; s < w->sims.size(); ++s) {
    if (mask && !mask[s]) continue;
    if (w->dirs[s].empty()) continue;
    const VtkSim& S = w->sims[s];
    const int k = w->next;
    w->next ^= 1;
    Slot& sl = w->slot[k];
    {
      std::unique_lock<std::mutex> lk(w->mu);
      w->cv.wait(lk, [&] { return !sl.busy; });
      sl.busy = true;
    }
    cudaError_t e = cudaSuccess;
    if (sl.copied_recorded) e = cudaStreamWaitEvent(w->stream, sl.copied, 0);
    if (e != cudaSuccess) {
      // without the wait the kernels could overwrite the slot while its previous copy still
      // reads it: return before launching anything into the slot
      std::lock_guard<std::mutex> lk(w->mu);
      sl.busy = false;
      err = std::string("vtk_write: ") + cudaGetErrorString(e);
      return -1;
    }
    const int64_t nb = beam_output_doubles(S.ne, w->pts);
    launch_beam_output(w->d, w->E, S.e0, S.ne, w->pts, sl.dev, w->stream);
    launch_node_output(w->d, S.n0, S.nn, sl.dev + nb, w->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(sl.ready, w->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(w->copy, sl.ready, 0);
    const size_t bytes = sizeof(double) * (size_t)(nb + node_output_doubles(S.nn));
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.host, sl.dev, bytes, cudaMemcpyDeviceToHost, w->copy);
    if (e == cudaSuccess) e = cudaEventRecord(sl.copied, w->copy);
    if (e != cudaSuccess) {
      std::lock_guard<std::mutex> lk(w->mu);
      sl.busy = false;
      err = std::string("vtk_write: ") + cudaGetErrorString(e);
      return -1;
    }
    sl.copied_recorded = true;
    {
      std::lock_guard<std::mutex> lk(w->mu);
      w->queue.push_back(Job{k, (int)s, counter ? counter[s] : 0, step ? step[s] : 0, t ? t[s] : 0.0});
      ++w->pending;
    }
    w->cv.notify_all();
  }
  return 0;
}

int vtk_flush(VtkWriter* w, std::string& err) {
  std::unique_lock<std::mutex> lk(w->mu);
  w->cv.wait(lk, [&] { return w->pending == 0; });
  if (!w->error.empty()) {
    err = w->error;
    w->error.clear();
    return -1;
  }
  return 0;
}

int vtk_close(VtkWriter* w, std::string& err) {
  int rc = vtk_flush(w, err);
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->stop = true;
  }
  w->cv.notify_all();
  if (w->th.joinable()) w->th.join();
  // paraview_collection (visualization_beams.jl:66-67): both files of each write under its time
  for (size_t s = 0; s < w->sims.size(); ++s) {
    if (w->dirs[s].empty()) continue;
    const std::string path = w->dirs[s] + "/simulation.pvd";
    FILE* fp = std::fopen(path.c_str(), "w");
    if (!fp) {
      if (rc == 0) err = "cannot open " + path + ": " + std::strerror(errno);
      rc = -1;
      continue;
    }
    std::fprintf(fp, "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n");
    std::fprintf(fp, "<VTKFile type=\"Collection\" version=\"1.0\" byte_order=\"LittleEndian\">\n  <Collection>\n");
    for (const PvdEntry& p : w->pvd[s]) {
      std::fprintf(fp, "    <DataSet timestep=\"%.17g\" part=\"0\" file=\"%s\"/>\n", p.t, p.beams.c_str());
      std::fprintf(fp, "    <DataSet timestep=\"%.17g\" part=\"1\" file=\"%s\"/>\n", p.t, p.nodes.c_str());
    }
    std::fprintf(fp, "  </Collection>\n</VTKFile>\n");
    if (std::fclose(fp) != 0 && rc == 0) {
      err = "write failed: " + path;
      rc = -1;
    }
  }
  cudaStreamSynchronize(w->copy ? w->copy : w->stream);
  w->free_all();
  delete w;
  return rc;
}

}  // namespace eb
