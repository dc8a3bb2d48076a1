// Host-side data structures and prep algorithms of the GB300 matrix powers
// kernel (MPK).  Everything here is plain C++17 and runs on the CPU; the
// CUDA side (device.cu) consumes the plans built here.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pdmpk_gb300.h"

namespace mpkg {

// Status codes shared with the C ABI (include/mpk_gb300.h).
enum Status : int {
  kOk = 0,
  kEInval = -1,
  kEIo = -2,
  kEFormat = -3,
  kEStruct = -4,
  kECuda = -5,
  kETimeout = -6,
  kENoMem = -7,
  kERange = -8,
};

// Records an error message for the calling thread and returns `code`.
int fail(int code, const std::string &msg);
const char *last_error();
void clear_error();

// Compressed sparse rows, 0-based, int32 indices (the reference's crs0_t
// plus optional values).
struct Csr {
  int n = 0;
  std::vector<int> ptr;     // n + 1
  std::vector<int> col;     // ptr[n]
  std::vector<double> val;  // empty => 1/deg operator
  long nnz() const { return ptr.empty() ? 0 : ptr[n]; }
};

// ---- graph input / output (graph.cc) ---------------------------------
// METIS text graph: header "n ne", one line per vertex with 1-based
// neighbours (the format read by mpk2/lib.c:69-129 read_crs).
int read_metis(const std::string &path, Csr *g, long *ne_header = nullptr);
int write_metis(const std::string &path, const Csr &g, long ne_header);
// Whitespace separated values, CSR order (mpk2/comm_data.c:160-187).
int read_values(const std::string &path, long nnz, std::vector<double> *val);
int write_values(const std::string &path, const std::vector<double> &val);
// Matrix Market (coordinate real/pattern, general/symmetric), with the
// semantics of pdmpk/csr.cc:9-122 (pattern => 1/deg values).
int read_mtx(const std::string &path, Csr *g);

// ---- generators (graph.cc) -------------------------------------------
// The reference stencil generators' graphs (mpk2/gen2.c:59-267):
// type in {m5p, t5p, m7p, m9p, cube}, values as gen2 writes them.
int gen_reference_stencil(const std::string &type, int size, Csr *g);
// d-dimensional Laplacian with 2d+1 points per interior row on an
// nx*ny*nz grid (nz = 1 for 2-D), columns ascending, diagonal `diag`,
// off-diagonals `off`.  Grid coordinates (x fastest) go to `coords`
// when non-null (3 ints per vertex).
int gen_laplacian(int nx, int ny, int nz, double diag, double off, Csr *g,
                  std::vector<int> *coords);
// Variable-coefficient diffusion operators with log-normal edge
// coefficients c_e = exp(sigma * N(0,1)) (seeded), symmetric, off-diagonal
// -w_d c_e, diagonal (1 + dominance) * sum of |off-diagonals|, columns
// ascending.  9-point on nx*ny (direction weights wx, wy, wdiag) and
// 7-point on nx*ny*nz (wx = wy = wz = 1).
int gen_diffusion_9pt(int nx, int ny, double sigma, double wx, double wy, double wdiag, double dominance,
                      uint64_t seed, Csr *g);
int gen_diffusion_7pt(int nx, int ny, int nz, double sigma, double dominance, uint64_t seed, Csr *g);
// Random banded, diagonally dominant operator (see graph.cc).
int gen_banded(long n, int bw, int nmin, int nmax, uint64_t seed, Csr *g);
// Uniform[-1, 1] doubles from a splitmix64 stream (seeded).
void uniform_vector(uint64_t seed, long n, double *out);

// ---- partitions (partition.cc) ----------------------------------------
// gpmetis output format: one part id per line (mpk2/lib.c:273-284).
int read_partition(const std::string &path, int n, std::vector<int> *part, int *npart);
int write_partition(const std::string &path, const std::vector<int> &part);
// Recursive coordinate bisection on integer grid coordinates.
int partition_rcb(int n, const std::vector<int> &coords, int dim, int npart,
                  std::vector<int> *part);
// Graph-only recursive bisection: breadth-first growth from a
// pseudo-peripheral vertex, halves by BFS order.  Works on any graph.
int partition_bfs(const Csr &g, int npart, std::vector<int> *part);
// METIS (when the build links it; see partition.cc).  Option slots of the
// METIS 5.1 layout this library sets.
constexpr int kMetisNOptions = 40, kMetisOptUfactor = 16, kMetisOptNumbering = 17;
bool have_metis();
// METIS_PartGraphKway on the graph exactly as given (options: null or
// kMetisNOptions values, -1 = METIS's default).
int metis_kway(int n, const int *ptr, const int *col, const int *vwgt, const int *adjwgt, int npart,
               const int *options, int *part, long *edgecut);
// gpmetis -ufactor=<ufactor> on g (self loops dropped; ufactor <= 0: METIS's
// default imbalance).
int partition_metis(const Csr &g, const int *vwgt, const int *adjwgt, int npart, int ufactor, std::vector<int> *part,
                    long *edgecut);

// ---- levels, weights, skirts (prep.cc) ---------------------------------
// comp_level / update_level (mpk2/lib.c:330-412): level_org == nullptr for
// the first phase.
int comp_levels(const Csr &g, const std::vector<int> &part, int npart,
                const std::vector<int> *level_org, std::vector<int> *level);
// level2wcrs (mpk2/lib.c:504-537).
void level_weights(const Csr &g, const std::vector<int> &level, std::vector<int> *wv,
                   std::vector<int> *we);
int write_weighted_graph(const std::string &path, const Csr &g, const std::vector<int> &we);
int write_levels(const std::string &path, const std::vector<int> &level);
int read_levels(const std::string &path, int n, std::vector<int> *level);

// Sparse skirt of one part: vertices (ascending ids) with their graph
// distance to the part, only those the skirt file keeps.
struct PartSkirt {
  std::vector<int> vert;
  std::vector<int> dist;
};
// Bounded BFS distances to each part, keeping dist < level (PA1, lev ==
// nullptr) or lev[j] < level - dist (after phases), exactly the entries
// that write_skirt (mpk2/lib.c:617-654) prints.
int comp_skirts(const Csr &g, const std::vector<int> &part, int npart,
                const std::vector<int> *lev, int level, std::vector<PartSkirt> *sk);
int write_skirt_file(const std::string &path, int n, int level,
                     const std::vector<PartSkirt> &sk);
int read_skirt_file(const std::string &path, int n, int npart, int level,
                    std::vector<PartSkirt> *sk);

// ---- task lists (prep.cc) ----------------------------------------------
// The (phase, part) task lists of prep_mpk (mpk2/mpkprep.c:7-258): list t =
// phase*npart + part holds entries l*n+i in [off[t], off[t+1]),
// level-major, vertex-ascending.
struct TaskLists {
  int n = 0, npart = 0, nlevel = 0, nphase = 0;
  std::vector<long> off;
  std::vector<long> idx;
};
// parts: max(nphase,1) partitions; levels: nphase level arrays; skirt per
// part of the phase-0 partition.  `check` runs the reference's dependency
// checks and returns kEStruct when they fail.
int build_tasks(const Csr &g, int npart, int nlevel, int nphase,
                const std::vector<std::vector<int>> &parts,
                const std::vector<std::vector<int>> &levels,
                const std::vector<PartSkirt> &sk, bool check, TaskLists *tl);

// ---- PA1 tile plans (prep.cc) -------------------------------------------
// One tile per part: the part plus its (nlevel)-deep halo, slots ordered by
// (distance, vertex id), so level l is computed on the prefix of slots with
// distance <= nlevel - l.
struct TilePlan {
  int n = 0, npart = 0, nlevel = 0;
  std::vector<int> order;          // part ids in launch order
  std::vector<long> slot_off;      // per tile: first slot (npart + 1)
  std::vector<int> shell;          // per tile: (nlevel + 1) prefix counts c_d
  std::vector<int> slot_vert;      // global vertex of each slot
  // Sliced-ELL (32 rows per slice) local structure of the rows with
  // distance <= nlevel - 1: column = local slot, 0xFFFF = padding.
  std::vector<long> slice_off;     // per tile: first slice (npart + 1)
  std::vector<long> ell_off;       // per slice: first entry (nslices + 1)
  std::vector<uint16_t> ell_col;
  std::vector<uint8_t> ell_width;  // per slice
  int max_slots = 0;               // largest c_nlevel
  long total_rows = 0;             // sum over levels of rows computed
};
int build_tile_plan(const Csr &g, const std::vector<int> &part, int npart, int nlevel,
                    TilePlan *tp);
// Tile launch order: breadth-first over the part graph (neighbouring tiles
// consecutive, so shared halo rows are reused from L2).
void part_order(const Csr &g, const std::vector<int> &part, int npart, std::vector<int> *order);
// The same plan built on the current GPU (prep_gpu.cu); falls back to
// build_tile_plan for balls beyond its capacity and for every error case.
// *on_gpu tells which ran.
int build_tile_plan_gpu(const Csr &g, const std::vector<int> &part, int npart, int nlevel,
                        TilePlan *tp, bool *on_gpu);
// PA1 task lists (nphase = 0: comp_skirts + build_tasks without the
// dependency checks) built on the current GPU, with the same fallback.
int build_pa1_tasks_gpu(const Csr &g, const std::vector<int> &part, int npart, int nlevel,
                        TaskLists *tl, bool *on_gpu);

// ---- level pipeline plans (prep.cc) ---------------------------------------
// Zero-redundancy pipeline: rows in chunks of `chunk` consecutive ids;
// chunk c at level l waits for chunks dep_lo[c]..dep_hi[c] at level l-1.
struct PipePlan {
  int n = 0, nlevel = 0, chunk = 0, nchunk = 0;
  std::vector<int> dep_lo, dep_hi;
  int reach = 0;  // max chunk distance of a dependency
};
int build_pipe_plan(const Csr &g, int nlevel, int chunk, PipePlan *pp);

// ---- MPI-2 rank buffers (bufs.cc) ----------------------------------------
// One rank's computation/communication buffers, the layout of buffers_t
// (mpk2/buffers.h:18-100): per phase an rbuf (received values, phase 0 =
// the x halo) followed by an mbuf (values computed by this rank),
// tile-local CSR mptr/mcol whose columns index the rank's own vv_buf, the
// send list idx_sbuf, and MPI counts/displacements per phase.
struct RankBuffers {
  int n = 0, npart = 0, nlevel = 0, nphase = 0, rank = 0;
  int buf_count = 0, buf_scount = 0, mptr_count = 0, mcol_count = 0;
  std::vector<int> recvcounts, sendcounts, rdispls, sdispls;  // npart*(nphase+1)
  std::vector<int> rcount, mcount, scount, rbuf_offsets, mbuf_offsets, sbuf_offsets, mptr_offsets,
      mcol_offsets;                                          // nphase+1
  std::vector<long> idx_buf, idx_sbuf, mptr_buf, mcol_buf;
  std::vector<double> mval_buf;  // empty when the file holds no values
};
// rank<N>.bufs as write_buffers writes it (mpk2/buffers.c:588-631).
int read_rank_buffers(const std::string &path, RankBuffers *b);
int write_rank_buffers(const std::string &path, const RankBuffers &b);
// Checks the internal consistency of a set of rank buffers (counts,
// offsets, index ranges, matching send/receive counts).
int check_rank_buffers(const std::vector<RankBuffers> &bufs);
// The MPI-2 prep of every rank (fill_buffers + alloc_fill_mval,
// mpk2/buffers.c:573-586, mpk2/mpi2_mpkwrtbufs.c:12-29), computed for all
// ranks at once with sparse communication sets instead of the reference's
// dense level*n*P*P table.  g: the matrix with values (loop.g0 +
// .loop.val); parts: max(nphase,1) partitions (relabelled in place for
// phases > 0, as reduce_comm does); levels: nphase level arrays; sk: the
// skirt of every part as read from s<nphase>.
int fill_all_buffers(const Csr &g, int npart, int nlevel, int nphase, std::vector<std::vector<int>> *parts,
                     const std::vector<std::vector<int>> &levels, const std::vector<PartSkirt> &sk,
                     std::vector<RankBuffers> *out);
// pdmpk buffers of all ranks flattened for one-GPU execution: one global
// mbuf (ranks concatenated), per batch a communication gather (the
// batch's MPI_Ialltoallv) and the batch's rows (seed + CSR terms), and
// the input/result scatters (Buffers::LoadInput, Results::FillResults).
struct PdExecMaps {
  int n = 0, nlevel = 0, nbatch = 0;
  long mbuf_total = 0;
  std::vector<long> in_dst, in_src;          // mbuf[in_dst] = x[in_src]
  std::vector<long> cm_dst, cm_src, cm_off;  // per batch (nbatch + 1 offsets)
  std::vector<long> row_off;                 // per batch (nbatch + 1)
  std::vector<long> row_dst, row_init, row_ptr, gcol;  // row_init -1: no seed
  std::vector<double> gval;
  std::vector<long> out_src, out_dst;        // y[out_dst] = mbuf[out_src]
};
int pd_exec_maps(const std::vector<pdmpk_gb300::Buffers> &bufs, PdExecMaps *m);

// Linear assignment maximising the trace: perm[j] = row assigned to column
// j of the npart x npart matrix sums (row-major).
void assign_max_trace(const std::vector<long> &sums, int npart, std::vector<int> *perm);

}  // namespace mpkg
