// pdmpk-compatible C++ interface of libmpk_gb300.so.
//
// The reference pdmpk (vatai/mpk, pdmpk/) is a C++ library: a prep program
// (apps/prep.cc) builds per-rank buffers with CommCompPatterns and dumps
// them as <name>-r<rank>-...buf.bin / results.bin; an MPI program
// (apps/exec.cc) loads them, one rank per part, and runs Buffers::AsyncExec.
// This header keeps the reference's class names, public fields and their
// meaning, and the on-disk format, so that buffers move between the two
// unchanged.  Execution differs by design: all ranks' buffers run on one
// GPU in one plan (mpkg_plan_pdmpk), the MPI_Ialltoallv of every batch
// becomes a device gather, and nothing here executes SpMV on the CPU.
//
// Errors: the reference throws std::logic_error (Csr) or exits; here the
// functions return the status codes of mpk_gb300.h (text with
// mpkg_last_error()), and only the Csr constructor throws, as the
// reference's does.
#ifndef PDMPK_GB300_H
#define PDMPK_GB300_H

#include <cstddef>
#include <functional>
#include <string>
#include <utility>
#include <vector>

namespace pdmpk_gb300 {

typedef int idx_t;                          // METIS idx_t, 32-bit (pdmpk/typedefs.h)
typedef short level_t;                      // pdmpk/typedefs.h:13
typedef std::pair<idx_t, idx_t> sidx_tidx_t;  // pdmpk/typedefs.h:15

// pdmpk/phased_vector.hpp:11-25: a vector with the start of every batch.
template <typename T>
class phased_vector : public std::vector<T> {
 public:
  std::vector<size_t> phase_begin;
  void rec_phase_begin() { phase_begin.push_back(this->size()); }
  T *get_ptr(const int &phase) { return this->data() + phase_begin[phase]; }
};

// pdmpk/phase_descriptor.h:11-38: levels [bottom, top) computed in a phase;
// batches below `mid` wait for their communication before computing.
// Serialised as three shorts.
class PhaseDescriptor {
 public:
  PhaseDescriptor() : bottom(-1), mid(0), top(-1) {}
  void UpdateBottom(const level_t &lbelow) {
    if (bottom == -1) bottom = mid = lbelow;
  }
  void UpdateMid(const level_t &lbelow) {
    if (mid <= lbelow) mid = (level_t)(lbelow + 1);
  }
  void UpdateTop(const level_t &lbelow) {
    if (top <= lbelow) top = (level_t)(lbelow + 1);
  }
  level_t bottom, mid, top;
};

// pdmpk/csr.h:11-69.  The constructor reads a Matrix Market file
// (coordinate, real or pattern, general or symmetric; pattern => 1/deg
// values) and throws std::logic_error on a bad banner or a non-square
// matrix, as the reference.  Symmetric files give a consistent CSR here
// (the reference counts only the stored triangle in `ptr`).
class Csr {
 public:
  Csr() = default;
  explicit Csr(const std::string &fname);
  // MPK gold on the GPU (k chained SpMVs, CSR order, separate multiply and
  // add as the reference's Csr::SpMV): vec <- A^nlevels vec.
  int MPK(const int &nlevels, std::vector<double> &vec) const;
  idx_t n = 0, nnz = 0;
  std::vector<idx_t> ptr, col;
  std::vector<double> val;
  bool pattern = false, symmetric = false;
};

// pdmpk/mcsr.h:14-39: the rank's rows, columns index the rank's mbuf.
class Mcsr {
 public:
  size_t MptrSize(const int &phase) const { return mptr.phase_begin[phase + 1] - mptr.phase_begin[phase]; }
  void NextMcolIdxToMptr() { mptr.push_back((idx_t)mcol.size()); }
  phased_vector<idx_t> mptr;
  std::vector<idx_t> mcol;
  std::vector<double> mval;
};

// pdmpk/mpi_buffers.h:15-72: per batch `npart` counts/displacements,
// the send list and the partial-row seeds (mbuf source, mbuf target).
class MpiBuffers {
 public:
  explicit MpiBuffers(const idx_t &npart) : npart(npart) {}
  void PhaseInit();
  void FillDispls();
  void SortInitIdcs();
  size_t SbufSize(const int &phase) const;
  size_t RbufSize(const int &phase) const;
  std::vector<int> sendcounts, sdispls, recvcounts, rdispls;
  phased_vector<idx_t> sbuf_idcs;
  phased_vector<sidx_tidx_t> init_idcs;
  idx_t npart;
};

// pdmpk/results.h:15-65: where each of the rank's results lives.
class Results {
 public:
  void SaveIndex(const idx_t &idx, const idx_t &mbuf_idx) {
    original_idcs.push_back(idx);
    mbuf_idcs.push_back(mbuf_idx);
  }
  std::vector<idx_t> original_idcs;  // matrix row of each result
  std::vector<idx_t> mbuf_idcs;      // its slot in mbuf
  std::vector<double> values;        // empty after prep
};

// pdmpk/buffers.h:30-166: one rank's buffers.  `mbuf` carries only the
// batch starts on the host (its values live on the GPU).
class Buffers {
 public:
  explicit Buffers(const idx_t &npart) : mpi_bufs(npart) {}
  // Reads / writes the reference's buf.bin + results.bin pair
  // (pdmpk/buffers.cc:194-224, pdmpk/results.cc:36-46).
  int Load(const std::string &buf_bin, const std::string &results_bin);
  int Dump(const std::string &buf_bin, const std::string &results_bin) const;
  int GetNumPhases() const { return (int)mbuf.phase_begin.size(); }
  void PreBatch();
  void PostBatch(const int &batch);

  MpiBuffers mpi_bufs;
  Mcsr mcsr;
  std::vector<PhaseDescriptor> phase_descriptors;
  size_t max_sbuf_size = 0;
  idx_t mbuf_idx = 0;
  phased_vector<double> mbuf;
  std::vector<idx_t> home_idcs;      // SendHome: mbuf[i] = mbuf[home_idcs[i]]
  std::vector<idx_t> original_idcs;  // LoadInput: matrix row of mbuf[i], i < mbuf.phase_begin[0]
  Results results;
};

// The file name the reference gives a rank's file (pdmpk/args.cc:199-213,
// default METIS options): <mtx>-np<P>-nl<L>-mm<M>-wm<W>[-r<rank>]-<branch>-<hash>.<suffix>
std::string Filename(const std::string &mtxname, int npart, int nlevel, int mirror_method, int weight_update_method,
                     int rank, const std::string &branch, const std::string &hash, const std::string &suffix);

// Partition provider behind pdmpk's two METIS call sites
// (pdmpk/pdmpk_buffers.cc:182-201).  `call` counts the calls of one prep
// (0 = the initial partition); `adjwgt` is null for call 0, else the edge
// weights of the active weight_update_method.  Returns 0 on success.
typedef std::function<int(const Csr &csr, const idx_t *adjwgt, int npart, int call, idx_t *part)> Partitioner;
// Contiguous blocks shifted by half a block per call: part of i =
// ((i + call*n/(2*npart)) mod n) * npart / n.
Partitioner BlockShiftPartitioner();
// Breadth-first recursive bisection of the graph (weights ignored).
Partitioner BfsPartitioner();
// METIS_PartGraphKway exactly as the reference calls it
// (pdmpk/pdmpk_buffers.cc:183-202): the CSR pattern as is (diagonal
// included), no vertex weights, the edge weights on calls after the first,
// default options (none on the first call).  Fails when the library was
// built without METIS.
Partitioner MetisPartitioner();

// pdmpk/args.h: the prep parameters.
struct Args {
  int npart = 0, nlevel = 0;
  int mirror_method = 0;         // 0..5: pdmpk/comm_comp_patterns.cc ProcAllPhases0..5
  int weight_update_method = 0;  // 0..3: pdmpk/pdmpk_buffers.cc UpdateWeights0..3
  Partitioner partitioner;       // BlockShiftPartitioner() when empty
};

// CommCompPatterns (pdmpk/comm_comp_patterns.cc:26-768): the pdmpk prep of
// every rank.  kEStruct when the mirror strategy cannot finish (the
// reference exits there).
int CommCompPatterns(const Csr &csr, const Args &args, std::vector<Buffers> *bufs);

}  // namespace pdmpk_gb300

#endif
