/*
 * Single-rank MPI stand-in used only to compile and link the reference
 * Dendro-KT sources as a CPU oracle.  Test infrastructure: nothing in the
 * product links against this file.
 *
 * Semantics: one process, rank 0 of size 1.  Collectives copy the send buffer
 * to the receive buffer.  Point-to-point messages to self are queued in FIFO
 * order per (tag) and matched by MPI_Recv / MPI_Irecv + MPI_Wait.  Datatypes
 * are represented by their byte size, which is all single-rank copy semantics
 * need.  Only the subset of MPI the reference calls is provided.
 */
#ifndef DKT_ORACLE_MPI_SHIM_H
#define DKT_ORACLE_MPI_SHIM_H

#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;   /* byte size of one element */
typedef int MPI_Op;
typedef int MPI_Group;
typedef int MPI_Request;
typedef void (MPI_User_function)(void *, void *, int *, MPI_Datatype *);

struct MPI_Status { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; int count; };

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 1
#define MPI_COMM_NULL 0
#define MPI_UNDEFINED (-32766)
#define MPI_SUCCESS 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *) 0)
#define MPI_STATUSES_IGNORE ((MPI_Status *) 0)
#define MPI_REQUEST_NULL (-1)
#define MPI_IN_PLACE ((void *) 1)

#define MPI_BYTE ((MPI_Datatype) 1)
#define MPI_CHAR ((MPI_Datatype) sizeof(char))
#define MPI_UNSIGNED_CHAR ((MPI_Datatype) sizeof(unsigned char))
#define MPI_SHORT ((MPI_Datatype) sizeof(short))
#define MPI_UNSIGNED_SHORT ((MPI_Datatype) sizeof(unsigned short))
#define MPI_INT ((MPI_Datatype) sizeof(int))
#define MPI_UNSIGNED ((MPI_Datatype) sizeof(unsigned))
#define MPI_LONG ((MPI_Datatype) sizeof(long))
#define MPI_UNSIGNED_LONG ((MPI_Datatype) sizeof(unsigned long))
#define MPI_LONG_LONG_INT ((MPI_Datatype) sizeof(long long))
#define MPI_LONG_LONG ((MPI_Datatype) sizeof(long long))
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype) sizeof(unsigned long long))
#define MPI_FLOAT ((MPI_Datatype) sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype) sizeof(double))
#define MPI_LONG_DOUBLE ((MPI_Datatype) sizeof(long double))

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROD 4
#define MPI_LAND 5
#define MPI_LOR 6

namespace dkt_mpi_shim {
struct Msg { int tag; std::vector<char> data; };
struct PendingRecv { void *buf; int bytes; int tag; bool active; };
inline std::deque<Msg> &queue() { static std::deque<Msg> q; return q; }
inline std::vector<PendingRecv> &pending() { static std::vector<PendingRecv> p; return p; }
inline bool take(int tag, void *buf, int bytes) {
  auto &q = queue();
  for (auto it = q.begin(); it != q.end(); ++it) {
    if (tag == MPI_ANY_TAG || it->tag == tag) {
      int n = (int) it->data.size() < bytes ? (int) it->data.size() : bytes;
      if (n > 0) std::memcpy(buf, it->data.data(), n);
      q.erase(it);
      return true;
    }
  }
  return false;
}
inline void put(int tag, const void *buf, int bytes) {
  Msg m; m.tag = tag; m.data.resize(bytes > 0 ? bytes : 0);
  if (bytes > 0) std::memcpy(m.data.data(), buf, bytes);
  queue().push_back(m);
}
inline void copy(const void *s, void *r, int bytes) {
  if (s == MPI_IN_PLACE || s == r || bytes <= 0) return;
  std::memmove(r, s, bytes);
}
}  // namespace dkt_mpi_shim

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Comm_free(MPI_Comm *) { return 0; }
inline int MPI_Comm_group(MPI_Comm, MPI_Group *g) { *g = 1; return 0; }
inline int MPI_Group_incl(MPI_Group, int n, const int *, MPI_Group *g) { *g = n; return 0; }
inline int MPI_Group_free(MPI_Group *) { return 0; }
inline int MPI_Comm_create(MPI_Comm c, MPI_Group g, MPI_Comm *nc) { *nc = (g > 0 ? c : MPI_COMM_NULL); return 0; }
inline int MPI_Comm_split(MPI_Comm c, int color, int, MPI_Comm *nc) { *nc = (color == MPI_UNDEFINED ? MPI_COMM_NULL : c); return 0; }
inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *nt) { *nt = count * old; return 0; }
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
inline int MPI_Type_free(MPI_Datatype *) { return 0; }
inline int MPI_Op_create(MPI_User_function *, int, MPI_Op *op) { *op = 100; return 0; }
inline int MPI_Op_free(MPI_Op *) { return 0; }

inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *r)
{ dkt_mpi_shim::put(tag, b, n * t); *r = MPI_REQUEST_NULL; return 0; }
inline int MPI_Issend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r)
{ return MPI_Isend(b, n, t, d, tag, c, r); }
inline int MPI_Send(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm)
{ dkt_mpi_shim::put(tag, b, n * t); return 0; }
inline int MPI_Recv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Status *)
{
  if (!dkt_mpi_shim::take(tag, b, n * t)) { std::fprintf(stderr, "mpi shim: recv with no matching send\n"); std::abort(); }
  return 0;
}
inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *r)
{
  auto &p = dkt_mpi_shim::pending();
  p.push_back({b, n * t, tag, true});
  *r = (int) p.size() - 1;
  return 0;
}
inline int MPI_Wait(MPI_Request *r, MPI_Status *)
{
  if (r == nullptr || *r == MPI_REQUEST_NULL) return 0;
  auto &p = dkt_mpi_shim::pending();
  if (*r >= 0 && *r < (int) p.size() && p[*r].active) {
    if (!dkt_mpi_shim::take(p[*r].tag, p[*r].buf, p[*r].bytes)) {
      std::fprintf(stderr, "mpi shim: wait on a receive with no matching send\n"); std::abort();
    }
    p[*r].active = false;
  }
  *r = MPI_REQUEST_NULL;
  return 0;
}
inline int MPI_Waitall(int n, MPI_Request *r, MPI_Status *)
{ for (int i = 0; i < n; i++) MPI_Wait(&r[i], nullptr); return 0; }
inline int MPI_Sendrecv(const void *sb, int sn, MPI_Datatype st, int, int, void *rb, int rn, MPI_Datatype rt, int, int, MPI_Comm, MPI_Status *)
{ int sbytes = sn * st, rbytes = rn * rt; dkt_mpi_shim::copy(sb, rb, sbytes < rbytes ? sbytes : rbytes); return 0; }

inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) { dkt_mpi_shim::copy(s, r, n * t); return 0; }
inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) { dkt_mpi_shim::copy(s, r, n * t); return 0; }
inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) { dkt_mpi_shim::copy(s, r, n * t); return 0; }
inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm) { dkt_mpi_shim::copy(s, r, sn * st); return 0; }
inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) { dkt_mpi_shim::copy(s, r, sn * st); return 0; }
inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *displs, MPI_Datatype rt, MPI_Comm)
{ dkt_mpi_shim::copy(s, (char *) r + (long) displs[0] * rt, sn * st); return 0; }
inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) { dkt_mpi_shim::copy(s, r, sn * st); return 0; }
inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r, const int *, const int *rd, MPI_Datatype rt, MPI_Comm)
{ dkt_mpi_shim::copy((const char *) s + (long) sd[0] * st, (char *) r + (long) rd[0] * rt, sc[0] * st); return 0; }
inline double MPI_Wtime() { return 0.0; }

#endif
