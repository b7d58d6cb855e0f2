// LATfield2.hpp -- single-rank stand-in for the LATfield2 v1.1 API surface that
// gevolution 1.2's gevolution.hpp and background.hpp use.  Written from the call
// sites (gevolution.hpp, main.cpp:213-246 and 372-879, ic_basic.hpp:1990-2259,
// Particles_gevolution.hpp:170); LATfield2 itself is not part of this project.
//
// TEST INFRASTRUCTURE ONLY: it lets the reference's own source compile so that
// the CPU restatement in oracle/gev_oracle.c can be checked against it.
//
// Conventions fixed here (the same ones gev_oracle.h documents):
//   * Lattice(3, N, halo 1); sites iterate x fastest; Site +/- dir steps into
//     the halo; updateHalo() copies periodic images into both halo layers.
//   * Field<T> stores components contiguously per component.
//   * the Fourier lattice has coord(0) = kx in [0, N/2], coord(1), coord(2) in
//     [0, N); k-space fields have no halo.
//   * Particles keep one std::list per cell in ascending ID order; updateVel
//     returns sqrt of the maximum callback value; moveParticles wraps positions
//     into [0,1) and relinks.
//   * *_comm folds the upper halo back in the order x, y, z.
#ifndef GEV_LATFIELD2_SHIM
#define GEV_LATFIELD2_SHIM

#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <list>
#include <vector>

#include "gev_oracle.h"

typedef double Real;

#define COUT std::cout

#define FFT_FORWARD 1
#define FFT_BACKWARD -1

namespace LATfield2 {

enum { symmetric = 1, unsymmetric = 0 };
// the reduction kinds moveParticles / updateVel accept for their outputs
enum { SUM = 1, MAX = 2, MIN = 4 };

class Imag {
 public:
  double re_, im_;
  Imag() : re_(0.), im_(0.) {}
  Imag(double r, double i) : re_(r), im_(i) {}
  double &real() { return re_; }
  double &imag() { return im_; }
  double real() const { return re_; }
  double imag() const { return im_; }
  Imag conj() const { return Imag(re_, -im_); }
  Imag operator+(const Imag &b) const { return Imag(re_ + b.re_, im_ + b.im_); }
  Imag operator-(const Imag &b) const { return Imag(re_ - b.re_, im_ - b.im_); }
  Imag operator-() const { return Imag(-re_, -im_); }
  Imag operator*(const Imag &b) const { return Imag(re_ * b.re_ - im_ * b.im_, re_ * b.im_ + im_ * b.re_); }
  Imag operator*(double d) const { return Imag(re_ * d, im_ * d); }
  Imag operator/(double d) const { return Imag(re_ / d, im_ / d); }
  // complex quotient (a + bi)(c - di) / (c^2 + d^2): a convention of this shim
  Imag operator/(const Imag &b) const {
    const double n = b.re_ * b.re_ + b.im_ * b.im_;
    return Imag((re_ * b.re_ + im_ * b.im_) / n, (im_ * b.re_ - re_ * b.im_) / n);
  }
  Imag &operator+=(const Imag &b) { re_ += b.re_; im_ += b.im_; return *this; }
  Imag &operator-=(const Imag &b) { re_ -= b.re_; im_ -= b.im_; return *this; }
  Imag &operator*=(double d) { re_ *= d; im_ *= d; return *this; }
  Imag &operator/=(double d) { re_ /= d; im_ /= d; return *this; }
};
inline Imag operator*(double d, const Imag &a) { return Imag(d * a.re_, d * a.im_); }

class Lattice {
 public:
  int dim_, size_[3], halo_, fourier_;
  int skip_[2];
  Lattice() : dim_(3), halo_(0), fourier_(0) { size_[0] = size_[1] = size_[2] = 0; skip_[0] = skip_[1] = 0; }
  Lattice(int dim, const int *size, int halo) { initialize(dim, size, halo); }
  void initialize(int dim, const int *size, int halo) {
    dim_ = dim;
    for (int i = 0; i < 3; i++) size_[i] = size[i];
    halo_ = halo;
    fourier_ = 0;
    skip_[0] = skip_[1] = 0;
  }
  void initializeRealFFT(const Lattice &lat, int halo) {
    dim_ = 3;
    size_[0] = lat.size_[0] / 2 + 1;
    size_[1] = lat.size_[1];
    size_[2] = lat.size_[2];
    halo_ = halo;
    fourier_ = 1;
    skip_[0] = skip_[1] = 0;
  }
  int size(int i) const { return size_[i]; }
  int sizeLocal(int i) const { return size_[i]; }
  int halo() const { return halo_; }
  int *coordSkip() { return skip_; }
  long ext(int i) const { return size_[i] + 2 * halo_; }
  // one rank owns every site: the first and last site, x fastest
  long siteFirst() const { return 0; }
  long siteLast() const { return (long)size_[0] * size_[1] * size_[2] - 1; }
  long sitesGross() const { return ext(0) * ext(1) * ext(2); }
};

class Site {
 public:
  const Lattice *lat_;
  int c_[3];
  Site() : lat_(0) { c_[0] = c_[1] = c_[2] = 0; }
  Site(const Lattice &lat) : lat_(&lat) { c_[0] = c_[1] = c_[2] = 0; }
  void initialize(const Lattice &lat) { lat_ = &lat; c_[0] = c_[1] = c_[2] = 0; }
  void initialize(const Lattice &lat, long index) {
    lat_ = &lat;
    c_[0] = (int)(index % lat.size_[0]);
    c_[1] = (int)((index / lat.size_[0]) % lat.size_[1]);
    c_[2] = (int)(index / ((long)lat.size_[0] * lat.size_[1]));
  }
  void first() { c_[0] = c_[1] = c_[2] = 0; }
  bool test() const { return c_[2] < lat_->size_[2]; }
  void next() {
    if (++c_[0] < lat_->size_[0]) return;
    c_[0] = 0;
    if (++c_[1] < lat_->size_[1]) return;
    c_[1] = 0;
    ++c_[2];
  }
  int coord(int i) const { return c_[i]; }
  bool setCoord(int x, int y, int z) { c_[0] = x; c_[1] = y; c_[2] = z; return true; }
  Site operator+(int d) const { Site s(*this); s.c_[d] += 1; return s; }
  Site operator-(int d) const { Site s(*this); s.c_[d] -= 1; return s; }
  long index() const {
    const long h = lat_->halo_;
    return (c_[0] + h) + lat_->ext(0) * ((c_[1] + h) + lat_->ext(1) * (c_[2] + h));
  }
};

class rKSite : public Site {
 public:
  rKSite() {}
  rKSite(const Lattice &lat) : Site(lat) {}
};

template <class T>
class Field {
 public:
  Lattice *lat_;
  int ncomp_, rows_, cols_, sym_;
  std::vector<T> data_;
  Field() : lat_(0), ncomp_(0), rows_(0), cols_(0), sym_(0) {}
  void initialize(Lattice &lat, int nc = 1) {
    lat_ = &lat;
    ncomp_ = nc;
    rows_ = nc;
    cols_ = 1;
    sym_ = 0;
    data_.assign((size_t)ncomp_ * lat.sitesGross(), T());
  }
  void initialize(Lattice &lat, int rows, int cols, int symmetry) {
    lat_ = &lat;
    rows_ = rows;
    cols_ = cols;
    sym_ = symmetry;
    ncomp_ = symmetry == symmetric ? rows * (rows + 1) / 2 : rows * cols;
    data_.assign((size_t)ncomp_ * lat.sitesGross(), T());
  }
  Lattice &lattice() { return *lat_; }
  int components() const { return ncomp_; }
  int symmetry() const { return sym_; }
  int comp(int i, int j) const {
    if (!sym_) return i * cols_ + j;
    if (i > j) { int t = i; i = j; j = t; }
    static const int tab[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    return tab[i][j];
  }
  T &operator()(const Site &x) { return data_[(size_t)x.index()]; }
  T &operator()(const Site &x, int c) { return data_[(size_t)c * lat_->sitesGross() + x.index()]; }
  T &operator()(const Site &x, int i, int j) { return (*this)(x, comp(i, j)); }
  /* fill halo cells with periodic images */
  void updateHalo() {
    const int h = lat_->halo_;
    if (!h) return;
    const int N0 = lat_->size_[0], N1 = lat_->size_[1], N2 = lat_->size_[2];
    Site s(*lat_), t(*lat_);
    for (int c = 0; c < ncomp_; c++)
      for (int z = -h; z < N2 + h; z++)
        for (int y = -h; y < N1 + h; y++)
          for (int x = -h; x < N0 + h; x++) {
            if (x >= 0 && x < N0 && y >= 0 && y < N1 && z >= 0 && z < N2) continue;
            s.setCoord(x, y, z);
            t.setCoord((x + N0) % N0, (y + N1) % N1, (z + N2) % N2);
            (*this)(s, c) = (*this)(t, c);
          }
  }
  /* the upper-halo fold of the CIC projections, x then y then z */
  void foldUpperHalo() {
    const int N = lat_->size_[0];
    Site s(*lat_), t(*lat_);
    for (int c = 0; c < ncomp_; c++) {
      for (int z = 0; z <= N; z++)
        for (int y = 0; y <= N; y++) {
          s.setCoord(N, y, z); t.setCoord(0, y, z);
          (*this)(t, c) += (*this)(s, c);
        }
      for (int z = 0; z <= N; z++)
        for (int x = 0; x < N; x++) {
          s.setCoord(x, N, z); t.setCoord(x, 0, z);
          (*this)(t, c) += (*this)(s, c);
        }
      for (int y = 0; y < N; y++)
        for (int x = 0; x < N; x++) {
          s.setCoord(x, y, N); t.setCoord(x, y, 0);
          (*this)(t, c) += (*this)(s, c);
        }
    }
    for (size_t i = 0; i < data_.size(); i++) {
      /* clear the halo */
      long site = (long)(i % (size_t)lat_->sitesGross());
      long e0 = lat_->ext(0), e1 = lat_->ext(1);
      int x = (int)(site % e0) - 1, y = (int)((site / e0) % e1) - 1, z = (int)(site / (e0 * e1)) - 1;
      if (x < 0 || x >= N || y < 0 || y >= N || z < 0 || z >= N) data_[i] = T();
    }
  }
};

/* projection helpers (LATfield2) */
template <class T>
void projection_init(Field<T> *f) {
  for (size_t i = 0; i < f->data_.size(); i++) f->data_[i] = T();
}
inline void scalarProjectionCIC_comm(Field<Real> *f) { f->foldUpperHalo(); }
inline void vectorProjectionCICNGP_comm(Field<Real> *f) { f->foldUpperHalo(); }
inline void symtensorProjectionCICNGP_comm(Field<Real> *f) { f->foldUpperHalo(); }

/* r2c / c2r over the oracle's FFT; the backward transform preserves its input */
template <class C>
class PlanFFT {
 public:
  Field<Real> *r_;
  Field<C> *k_;
  PlanFFT(Field<Real> *r, Field<C> *k) : r_(r), k_(k) {}
  void execute(int dir) {
    const int N = r_->lat_->size_[0];
    const size_t V = (size_t)N * N * N, K = (size_t)N * N * (N / 2 + 1);
    std::vector<double> real(V), cplx(2 * K);
    Site x(*r_->lat_);
    for (int c = 0; c < r_->ncomp_; c++) {
      if (dir == FFT_FORWARD) {
        for (x.first(); x.test(); x.next())
          real[x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))] = (*r_)(x, c);
        gevo_fft_r2c(N, real.data(), cplx.data());
        memcpy(&k_->data_[(size_t)c * K], cplx.data(), sizeof(double) * 2 * K);
      } else {
        memcpy(cplx.data(), &k_->data_[(size_t)c * K], sizeof(double) * 2 * K);
        gevo_fft_c2r(N, cplx.data(), real.data());
        for (x.first(); x.test(); x.next())
          (*r_)(x, c) = real[x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))];
      }
    }
  }
};

/* particles */
struct part_simple {
  double pos[3];
  double vel[3];
  long ID;
};
struct part_simple_info {
  double mass;
  int relativistic;
  char type_name[64];
};
struct part_simple_dataType {};

template <class part>
struct CellList {
  std::list<part> parts;
  int size;
  CellList() : size(0) {}
};

template <class part>
class CellField {
 public:
  std::vector<CellList<part> > cells_;
  const Lattice *lat_;
  CellList<part> &operator()(const Site &x) {
    const int N = lat_->size_[0];
    return cells_[(size_t)x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))];
  }
};

template <class part, class part_info, class part_dataType>
class Particles {
 public:
  Lattice *lat_;
  double res_;
  part_info info_;
  CellField<part> field_;
  // the member names Particles_gevolution.hpp reads (its Gadget-2 writer and reader)
  Lattice lat_part_;
  double lat_resolution_;
  CellField<part> &field_part_;

  Particles() : lat_(0), res_(0.), lat_resolution_(0.), field_part_(field_) {}
  void initialize(part_info info, part_dataType, Lattice *lat, Real *) {
    info_ = info;
    lat_ = lat;
    res_ = 1.0 / (double)lat->size_[0];
    lat_part_ = *lat;
    lat_resolution_ = res_;
    field_.lat_ = lat;
    field_.cells_.assign((size_t)lat->size_[0] * lat->size_[1] * lat->size_[2], CellList<part>());
  }
  Lattice &lattice() { return *lat_; }
  double res() { return res_; }
  part_info *parts_info() { return &info_; }
  size_t mass_offset() { return offsetof(part_info, mass); }
  CellField<part> &field() { return field_; }

  long cellOf(const part &p) const {
    const int N = lat_->size_[0];
    return (long)gevo_cell_of(N, p.pos[0]) + (long)N * ((long)gevo_cell_of(N, p.pos[1]) + (long)N * gevo_cell_of(N, p.pos[2]));
  }
  static bool byID(const part &a, const part &b) { return a.ID < b.ID; }
  bool addParticle_global(const part &p) {
    CellList<part> &c = field_.cells_[(size_t)cellOf(p)];
    typename std::list<part>::iterator it = c.parts.begin();
    while (it != c.parts.end() && it->ID < p.ID) ++it;
    c.parts.insert(it, p);
    c.size++;
    return true;
  }
  /* rebuild all lists from the current positions (wrap, then ID order) */
  void relink() {
    std::vector<part> all;
    for (size_t i = 0; i < field_.cells_.size(); i++) {
      for (typename std::list<part>::iterator it = field_.cells_[i].parts.begin(); it != field_.cells_[i].parts.end(); ++it)
        all.push_back(*it);
      field_.cells_[i].parts.clear();
      field_.cells_[i].size = 0;
    }
    for (size_t i = 0; i < all.size(); i++) {
      for (int l = 0; l < 3; l++) gevo_wrap(&all[i].pos[l]);
      addParticle_global(all[i]);
    }
  }

  typedef Real (*vel_fn)(double, double, part *, double *, part_info, Field<Real> **, Site *, int, double *, double *, int);
  typedef void (*pos_fn)(double, double, part *, double *, part_info, Field<Real> **, Site *, int, double *, double *, int);

  struct MaxRed {
    double m;
    MaxRed() : m(0.) {}
    void operator()(Real v) { if (v > m) m = v; }
  };
  Real updateVel(vel_fn fn, double dtau, Field<Real> **fields, int nfield, double *params = NULL,
                 double *outputs = NULL, int * = NULL, int noutputs = 0) {
    for (int k = 0; k < nfield; k++) if (fields[k]) fields[k]->updateHalo();
    MaxRed r;
    Site x(*lat_);
    std::vector<Site> sites(nfield > 0 ? nfield : 1);
    for (x.first(); x.test(); x.next()) {
      CellList<part> &cl = field_(x);
      for (typename std::list<part>::iterator it = cl.parts.begin(); it != cl.parts.end(); ++it) {
        double ref_dist[3];
        for (int i = 0; i < 3; i++) ref_dist[i] = it->pos[i] / res_ - (double)x.coord(i);
        for (int k = 0; k < nfield; k++) {
          sites[k].initialize(fields[k] ? fields[k]->lattice() : *lat_);
          sites[k].setCoord(x.coord(0), x.coord(1), x.coord(2));
        }
        r(fn(dtau, res_, &(*it), ref_dist, info_, fields, sites.data(), nfield, params, outputs, noutputs));
      }
    }
    return std::sqrt(r.m);
  }
  void moveParticles(pos_fn fn, double dtau, Field<Real> **fields, int nfield, double *params = NULL,
                     double *outputs = NULL, int * = NULL, int noutputs = 0) {
    for (int k = 0; k < nfield; k++) if (fields[k]) fields[k]->updateHalo();
    Site x(*lat_);
    std::vector<Site> sites(nfield > 0 ? nfield : 1);
    for (x.first(); x.test(); x.next()) {
      CellList<part> &cl = field_(x);
      for (typename std::list<part>::iterator it = cl.parts.begin(); it != cl.parts.end(); ++it) {
        double ref_dist[3];
        for (int i = 0; i < 3; i++) ref_dist[i] = it->pos[i] / res_ - (double)x.coord(i);
        for (int k = 0; k < nfield; k++) {
          sites[k].initialize(fields[k] ? fields[k]->lattice() : *lat_);
          sites[k].setCoord(x.coord(0), x.coord(1), x.coord(2));
        }
        fn(dtau, res_, &(*it), ref_dist, info_, fields, sites.data(), nfield, params, outputs, noutputs);
      }
    }
    relink();
  }
};

/* scalarProjectionCIC_project (LATfield2): the CIC mass deposit m/dx^3 w of the
 * oracle (gevo_deposit_mass, which folds its own halo), added to the field */
template <class part, class part_info, class part_dataType>
void scalarProjectionCIC_project(Particles<part, part_info, part_dataType> *pcls, Field<Real> *rho) {
  const int N = pcls->lat_->size_[0];
  const size_t V = (size_t)N * N * N;
  std::vector<gevo_part> flat;
  std::vector<long> cs(V + 1, 0);
  for (size_t c = 0; c < V; c++) {
    cs[c] = (long)flat.size();
    for (typename std::list<part>::iterator it = pcls->field_.cells_[c].parts.begin();
         it != pcls->field_.cells_[c].parts.end(); ++it) {
      gevo_part q;
      for (int l = 0; l < 3; l++) {
        q.pos[l] = it->pos[l];
        q.vel[l] = it->vel[l];
      }
      q.ID = it->ID;
      flat.push_back(q);
    }
  }
  cs[V] = (long)flat.size();
  std::vector<double> out(V, 0.);
  gevo_deposit_mass(N, (long)flat.size(), flat.data(), cs.data(), pcls->info_.mass, out.data());
  Site x(rho->lattice());
  for (x.first(); x.test(); x.next())
    (*rho)(x) += out[x.coord(0) + (size_t)N * (x.coord(1) + (size_t)N * x.coord(2))];
}

}  // namespace LATfield2

#endif
