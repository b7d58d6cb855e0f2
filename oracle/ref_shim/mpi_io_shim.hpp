// mpi_io_shim.hpp -- single-rank stand-ins for the MPI-IO calls and the
// LATfield2 `parallel` object that Particles_gevolution.hpp's Gadget-2 writer
// and reader (Particles_gevolution.hpp:30-251, 574-665) and tools.hpp's spectra
// use.  Files are plain
// stdio; one rank owns the whole grid, so the rank-to-rank particle counts are a
// mailbox that a rank reads back from itself.
//
// TEST INFRASTRUCTURE ONLY: it lets the reference's own Gadget-2 code compile so
// that the CPU restatement in oracle/gev_oracle.c and the GPU path can be
// checked against it.
#ifndef GEV_MPI_IO_SHIM
#define GEV_MPI_IO_SHIM

#include <sys/types.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>

typedef long long MPI_Offset;
typedef int MPI_Status;
typedef int MPI_Comm;
typedef int MPI_Info;
typedef int MPI_Datatype;  // the element size in bytes
struct GevShimFile {
  FILE *f;
};
typedef GevShimFile *MPI_File;

#define MPI_MODE_WRONLY 1
#define MPI_MODE_CREATE 2
#define MPI_MODE_RDONLY 4
#define MPI_INFO_NULL 0
#define MPI_UNSIGNED 4
#define MPI_BYTE 1
#define MPI_FLOAT 4
#define MPI_SEEK_SET 0

// one rank: a reduction onto rank 0 in place leaves the buffer as it is
#define MPI_IN_PLACE ((void *)1)
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_SUM 0
inline int MPI_Reduce(const void *, void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }

inline int MPI_File_open(MPI_Comm, const char *name, int mode, MPI_Info, MPI_File *fh) {
  FILE *f = 0;
  if (mode & MPI_MODE_RDONLY)
    f = fopen(name, "rb");
  else {
    f = fopen(name, "r+b");
    if (!f && (mode & MPI_MODE_CREATE)) f = fopen(name, "w+b");
  }
  *fh = new GevShimFile;
  (*fh)->f = f;
  return f ? 0 : 1;
}
inline int MPI_File_close(MPI_File *fh) {
  if (*fh) {
    if ((*fh)->f) fclose((*fh)->f);
    delete *fh;
    *fh = 0;
  }
  return 0;
}
inline int MPI_File_set_size(MPI_File fh, MPI_Offset size) {
  if (!fh->f) return 1;
  fflush(fh->f);
  return ftruncate(fileno(fh->f), (off_t)size);
}
inline int MPI_File_write_at(MPI_File fh, MPI_Offset off, const void *buf, int count, MPI_Datatype t, MPI_Status *) {
  if (!fh->f || fseeko(fh->f, (off_t)off, SEEK_SET) != 0) return 1;
  return fwrite(buf, (size_t)t, (size_t)count, fh->f) == (size_t)count ? 0 : 1;
}
inline int MPI_File_write_at_all(MPI_File fh, MPI_Offset off, const void *buf, int count, MPI_Datatype t,
                                 MPI_Status *s) {
  return count > 0 ? MPI_File_write_at(fh, off, buf, count, t, s) : 0;
}
inline int MPI_File_read_all(MPI_File fh, void *buf, int count, MPI_Datatype t, MPI_Status *) {
  if (!fh->f) return 1;
  return fread(buf, (size_t)t, (size_t)count, fh->f) == (size_t)count ? 0 : 1;
}
inline int MPI_File_seek(MPI_File fh, MPI_Offset off, int) {
  return fh->f && fseeko(fh->f, (off_t)off, SEEK_SET) == 0 ? 0 : 1;
}

struct GevShimParallel {
  long long box_;
  int grank_[2], gsize_[2];
  MPI_Comm dim0_[1];
  GevShimParallel() : box_(0) {
    grank_[0] = grank_[1] = 0;
    gsize_[0] = gsize_[1] = 1;
    dim0_[0] = 0;
  }
  int rank() const { return 0; }
  int size() const { return 1; }
  bool isRoot() const { return true; }
  int *grid_rank() { return grank_; }
  int *grid_size() { return gsize_; }
  MPI_Comm lat_world_comm() const { return 0; }
  MPI_Comm *dim0_comm() { return dim0_; }
  template <class T>
  void send(T v, int) { box_ = (long long)v; }
  template <class T>
  void receive(T &v, int) { v = (T)box_; }
  template <class T>
  void send_dim0(T v, int) { box_ = (long long)v; }
  template <class T>
  void receive_dim0(T &v, int) { v = (T)box_; }
  template <class T>
  void broadcast_dim0(T &, int) {}
  template <class T>
  void broadcast(T &, int) {}
  template <class T>
  void broadcast_dim0(T *, long, int) {}
  template <class T>
  void broadcast(T *, long, int) {}
  void abortForce() { std::abort(); }
  void barrier() {}
  // one rank: reductions leave their operands as they are
  template <class T>
  void max(T &) {}
  template <class T>
  void sum(T &) {}
  template <class T>
  void sum(T *, int) {}
};
static GevShimParallel parallel;

#endif
