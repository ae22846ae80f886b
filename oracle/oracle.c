/*
 * oracle.c -- CPU restatement of LPMD's short-range MD timestep (see oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for libgbmd, never part of the product path.
 *
 * Every function names the reference lines it follows.  Arithmetic is written in the
 * reference's evaluation order (C++ left-to-right for chained * and +), and the file is
 * compiled with -ffp-contract=off so each product and sum rounds on its own, as in the
 * reference's x86-64 build.  Vector quantities are xyz-interleaved double[3n] arrays,
 * the layout of FixedSizeParticleSet (liblpmd/lpmd/fixedsizeparticleset.h:33-43).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_FORCEFACTOR 0.00964853 /* session string "0.00964853": liblpmd/runtime/session.cc:17-31 */
#define ORC_KIN2EV 103.64269       /* liblpmd/lpmd/properties.h:10 */
#define ORC_KBOLTZMANN 8.6173422E-05 /* liblpmd/lpmd/properties.h:11 */
#define ORC_PRESSFACTOR 160217.65  /* liblpmd/runtime/units.cc:9, "160217.65000000" */
#define ORC_MAXPOT 8

typedef struct {
  int kind;
  int spc_sum; /* Potential::SetValidSpecies: s1 + s2, negative = wildcard */
  double cutoff;
  double p[10];
  /* derived */
  double an, am;
  /* MetalPotential state: the per-atom density of the last force call */
  double* rho;
  /* FastLJ tables: etable[bins], fftable[bins] */
  double* tab;
  long bins;
} orc_pot;

typedef struct {
  int kind;
  double cutoff;
  /* linkedcell */
  int mode_auto, nx, ny, nz, side, cells_inside;
  int* head;
  int* tail;
  int64_t* atomlist;
  int64_t* indexc;
  int* subcell;
  double* cached_rcut_half; /* per-atom list cache, keyed on emptiness (see lc_list) */
  double* cached_rcut_full;
  int64_t last_atoms_size;
  /* verletlist */
  double extcut;
  int64_t maxneighbors, each, step_count, old_size;
  int64_t* nv;
  int64_t* vlist; /* n * maxneighbors */
  /* lcbinary: the atom of every sub-cell (-1: none) */
  int64_t* binlist;
} orc_cm;

struct orc_sim {
  int64_t n;
  double L[3];
  double* pos;
  double* vel;
  double* acc;
  double* old_acc; /* OldConfig().Atoms()[i].Acceleration() */
  int32_t* Z;
  double* mass;
  uint8_t* flags;
  int have_fixedvel, have_fixedpos;
  orc_cm* cm;
  orc_pot pots[ORC_MAXPOT];
  int npots;
  int have_integrator;
  int integ;       /* ORC_INT_* */
  double fmass, t0, friction; /* nosehoover */
  double* old_pos; /* OldConfig positions (verlet) */
  double* old_vel; /* OldConfig velocities (leapfrog) */
  double* aux;     /* the previous old acceleration (beeman, nosehoover) */
  double dt;
  int initialized;
  int64_t step;
  int64_t update_cell_calls;
  double energy[ORC_MAXPOT]; /* energycache per potential */
  double virial;
  double stress[3][3];
  /* scratch list for one atom */
  int64_t* lj;
  double* lrij;
  double* lr2;
  int64_t lcap;
};

/* ------------------------------------------------------------------------------------------- */
/* Geometry: OrthogonalCell (liblpmd/lpmd/orthogonalcell.h)                                     */
/* ------------------------------------------------------------------------------------------- */

/* OrthogonalCell::Displacement, orthogonalcell.h:131-149: d = b - a, one wrap per axis. */
void orc_displacement(const double L[3], const double a[3], const double b[3], double out[3]) {
  for (int q = 0; q < 3; ++q)
    out[q] = b[q] - a[q];
  for (int i = 0; i < 3; ++i) {
    double m = L[i];
    double mhalf = 0.5 * m;
    if (out[i] >= mhalf)
      out[i] -= m;
    else if (out[i] < -mhalf)
      out[i] += m;
  }
}

/* OrthogonalCell::FittedInside, orthogonalcell.h:102-114 (ll = v[q].Module() = sqrt(L*L)). */
void orc_fitted_inside(const double L[3], const double a[3], double out[3]) {
  for (int q = 0; q < 3; ++q) {
    double v = a[q];
    double ll = sqrt(L[q] * L[q]);
    if (v < 0.0)
      v -= ll * floor(v / ll);
    else if (v > ll)
      v -= ll * floor(v / ll);
    out[q] = v;
  }
}

/* Vector::SquareModule, liblpmd/lpmd/vector.h:107. */
static inline double sqmod(const double d[3]) { return d[0] * d[0] + d[1] * d[1] + d[2] * d[2]; }

/* ------------------------------------------------------------------------------------------- */
/* LinkedCell (plugins/linkedcell.cc)                                                          */
/* ------------------------------------------------------------------------------------------- */

/* WrapAround, linkedcell.cc:9-15. */
static inline int wrap_around(int i, int n) {
  if (i < 0)
    i += ((-i / n) + 1) * n;
  else if (i > n - 1)
    i -= (i / n) * n;
  return i;
}

/* Automatic subdivision, linkedcell.cc:146-204 (one axis). */
static int lc_auto_n(double len, double cutoff) {
  double fnn = (cutoff / 2.5);
  int n = 1;
  for (;;) {
    double previo = fabs(len / n - fnn);
    n++;
    double actual = fabs(len / n - fnn);
    if (actual < 1E-3)
      break;
    else if (actual > previo) {
      n--;
      break;
    }
  }
  if ((n % 2) != 0)
    n--;
  return n;
}

int orc_linkedcell_geometry(const double L[3], double cutoff, int nx, int ny, int nz, int mode_auto,
                            int* out_n, int* out_side, int* out_cells_inside) {
  if (mode_auto) {
    nx = lc_auto_n(L[0], cutoff);
    ny = lc_auto_n(L[1], cutoff);
    nz = lc_auto_n(L[2], cutoff);
  }
  if (nx <= 0 || ny <= 0 || nz <= 0)
    return ORC_ERR_INVALID; /* the reference divides by zero here */
  /* linkedcell.cc:216-222 */
  double d = L[0] / (double)nx;
  if (L[1] / (double)ny < d)
    d = L[1] / (double)ny;
  if (L[2] / (double)nz < d)
    d = L[2] / (double)nz;
  int side = (int)ceil((cutoff / d) - 0.5);
  out_n[0] = nx;
  out_n[1] = ny;
  out_n[2] = nz;
  *out_side = side;
  *out_cells_inside = (2 * side + 1) * (2 * side + 1) * (2 * side + 1);
  return ORC_OK;
}

static void cm_free(orc_cm* cm) {
  if (!cm)
    return;
  free(cm->head);
  free(cm->tail);
  free(cm->atomlist);
  free(cm->indexc);
  free(cm->subcell);
  free(cm->cached_rcut_half);
  free(cm->cached_rcut_full);
  free(cm->nv);
  free(cm->vlist);
  free(cm->binlist);
  free(cm);
}

/* LinkedCell::UpdateCell, linkedcell.cc:112-267.  The neighbour-list caches
 * (full_list_half/full_list_full) are cleared; see lc_list for how they are restated. */
static int lc_update_cell(orc_sim* s, orc_cm* cm) {
  const int64_t n = s->n;
  if (n != cm->last_atoms_size) {
    free(cm->atomlist);
    free(cm->indexc);
    free(cm->cached_rcut_half);
    free(cm->cached_rcut_full);
    cm->atomlist = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    cm->indexc = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    cm->cached_rcut_half = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    cm->cached_rcut_full = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!cm->atomlist || !cm->indexc || !cm->cached_rcut_half || !cm->cached_rcut_full)
      return ORC_ERR_NOMEM;
  }
  cm->last_atoms_size = n;
  if (cm->mode_auto) {
    cm->nx = lc_auto_n(s->L[0], cm->cutoff);
    cm->ny = lc_auto_n(s->L[1], cm->cutoff);
    cm->nz = lc_auto_n(s->L[2], cm->cutoff);
    cm->mode_auto = 0;
  }
  const int nx = cm->nx, ny = cm->ny, nz = cm->nz;
  if (nx <= 0 || ny <= 0 || nz <= 0)
    return ORC_ERR_INVALID;
  const int64_t ncell = (int64_t)nx * ny * nz;
  free(cm->head);
  free(cm->tail);
  cm->head = (int*)malloc(sizeof(int) * (size_t)ncell);
  cm->tail = (int*)malloc(sizeof(int) * (size_t)ncell);
  if (!cm->head || !cm->tail)
    return ORC_ERR_NOMEM;
  if (cm->subcell == NULL) {
    int nn[3], side, ci;
    orc_linkedcell_geometry(s->L, cm->cutoff, nx, ny, nz, 0, nn, &side, &ci);
    cm->side = side;
    cm->cells_inside = ci;
    cm->subcell = (int*)malloc(sizeof(int) * (size_t)(ncell * ci));
    if (!cm->subcell)
      return ORC_ERR_NOMEM;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          int r = 0;
          int64_t q = (int64_t)k * (nx * ny) + (int64_t)j * nx + i;
          for (int dz = -side; dz <= side; ++dz)
            for (int dy = -side; dy <= side; ++dy)
              for (int dx = -side; dx <= side; ++dx) {
                int z0 = wrap_around(i + dx, nx);
                int z1 = wrap_around(j + dy, ny);
                int z2 = wrap_around(k + dz, nz);
                int64_t p = (int64_t)z2 * (nx * ny) + (int64_t)z1 * nx + z0;
                cm->subcell[q * ci + (r++)] = (int)p;
              }
        }
  }
  for (int64_t q = 0; q < ncell; ++q)
    cm->head[q] = cm->tail[q] = -1;
  for (int64_t r = 0; r < n; ++r) {
    cm->cached_rcut_half[r] = -1.0;
    cm->cached_rcut_full[r] = -1.0;
    const double* x = &s->pos[3 * r];
    /* OrthogonalCell::Fractional: v[q] / modv[q] */
    double f0 = x[0] / s->L[0], f1 = x[1] / s->L[1], f2 = x[2] / s->L[2];
    int i = wrap_around((int)floor(nx * f0), nx);
    int j = wrap_around((int)floor(ny * f1), ny);
    int k = wrap_around((int)floor(nz * f2), nz);
    int64_t q = (int64_t)k * (nx * ny) + (int64_t)j * nx + i;
    cm->indexc[r] = (((q >= 0) && (q < ncell)) ? q : -1);
    q = cm->indexc[r];
    if (q >= 0) {
      if (cm->head[q] == -1)
        cm->head[q] = cm->tail[q] = (int)r;
      else {
        cm->atomlist[cm->tail[q]] = r;
        cm->tail[q] = (int)r;
      }
    }
    cm->atomlist[r] = -1;
  }
  return ORC_OK;
}

static int ensure_scratch(orc_sim* s, int64_t need) {
  if (need <= s->lcap)
    return ORC_OK;
  int64_t cap = s->lcap ? s->lcap : 256;
  while (cap < need)
    cap *= 2;
  int64_t* lj = (int64_t*)realloc(s->lj, sizeof(int64_t) * (size_t)cap);
  if (!lj)
    return ORC_ERR_NOMEM;
  s->lj = lj;
  double* lrij = (double*)realloc(s->lrij, sizeof(double) * 3 * (size_t)cap);
  if (!lrij)
    return ORC_ERR_NOMEM;
  s->lrij = lrij;
  double* lr2 = (double*)realloc(s->lr2, sizeof(double) * (size_t)cap);
  if (!lr2)
    return ORC_ERR_NOMEM;
  s->lr2 = lr2;
  s->lcap = cap;
  return ORC_OK;
}

static int push_pair(orc_sim* s, int64_t* cnt, int64_t z, const double rij[3], double r2) {
  if (*cnt >= s->lcap) {
    int rc = ensure_scratch(s, *cnt + 1);
    if (rc)
      return rc;
  }
  s->lj[*cnt] = z;
  s->lrij[3 * *cnt + 0] = rij[0];
  s->lrij[3 * *cnt + 1] = rij[1];
  s->lrij[3 * *cnt + 2] = rij[2];
  s->lr2[*cnt] = r2;
  (*cnt)++;
  return ORC_OK;
}

/* LinkedCell::BuildNeighborList, linkedcell.cc:293-360.
 * The reference caches each atom's half and full list until the next UpdateCell and only
 * rebuilds a list that is empty, so the first caller's rcut wins.  Positions do not change
 * between UpdateCell calls, so rebuilding with the remembered rcut yields the identical
 * list; that remembered rcut is what is stored here. */
static int lc_list(orc_sim* s, orc_cm* cm, int64_t i, int full, double rcut, int64_t* cnt) {
  *cnt = 0;
  int64_t cind = cm->indexc[i];
  if (cind < 0)
    return ORC_OK; /* atom outside the box: empty list (linkedcell.cc:304-311) */
  double* cache = full ? cm->cached_rcut_full : cm->cached_rcut_half;
  double rc = (cache[i] >= 0.0) ? cache[i] : rcut;
  const double* xi = &s->pos[3 * i];
  for (int c = 0; c < cm->cells_inside; ++c) {
    int neighbor_cell = cm->subcell[cind * cm->cells_inside + c];
    for (int64_t z = cm->head[neighbor_cell]; z != -1; z = cm->atomlist[z]) {
      if (z == i)
        continue;
      if ((full == 0) && (z > i))
        continue;
      double rij[3];
      orc_displacement(s->L, xi, &s->pos[3 * z], rij);
      double r2 = sqmod(rij);
      if (r2 < rc * rc) {
        int e = push_pair(s, cnt, z, rij, r2);
        if (e)
          return e;
      }
    }
  }
  if (*cnt > 0)
    cache[i] = rc;
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------------- */
/* VerletListCellManager (plugins/verletlist.cc)                                               */
/* ------------------------------------------------------------------------------------------- */

/* UpdateVerletList, verletlist.cc:67-104 (O(N^2), i < j, extcut^2 test). */
static int vl_rebuild(orc_sim* s, orc_cm* cm) {
  const int64_t n = s->n;
  if (fabs(cm->cutoff) < 1E-10)
    return ORC_ERR_INVALID; /* PluginError("verletlist", "No cutoff was defined") */
  if (n != cm->old_size || cm->nv == NULL) {
    free(cm->nv);
    free(cm->vlist);
    cm->nv = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    cm->vlist = (int64_t*)malloc(sizeof(int64_t) * (size_t)((n > 0 ? n : 1) * cm->maxneighbors));
    if (!cm->nv || !cm->vlist)
      return ORC_ERR_NOMEM;
  }
  for (int64_t i = 0; i < n; ++i)
    cm->nv[i] = 0;
  const double ext2 = cm->extcut * cm->extcut;
  const int64_t mx = cm->maxneighbors;
  for (int64_t i = 0; i < n - 1; ++i)
    for (int64_t j = i + 1; j < n; ++j) {
      double rij[3];
      orc_displacement(s->L, &s->pos[3 * i], &s->pos[3 * j], rij);
      if (sqmod(rij) < ext2) {
        if ((cm->nv[j] == mx - 1) || (cm->nv[i] == mx - 1))
          return ORC_ERR_MAXNEIGHBORS; /* "maxneighbors is too small!" */
        cm->vlist[j * mx + cm->nv[j]++] = i;
        cm->vlist[i * mx + cm->nv[i]++] = j;
      }
    }
  return ORC_OK;
}

/* VerletListCellManager::UpdateCell, verletlist.cc:124-131.  step_count counts calls. */
static int vl_update_cell(orc_sim* s, orc_cm* cm) {
  int mustupdate = (((cm->step_count % cm->each) == 0) || (s->n != cm->old_size));
  int rc = ORC_OK;
  if (mustupdate)
    rc = vl_rebuild(s, cm);
  cm->step_count++;
  cm->old_size = s->n;
  return rc;
}

/* VerletListCellManager::BuildNeighborList, verletlist.cc:135-167 (half list keeps j > i). */
static int vl_list(orc_sim* s, orc_cm* cm, int64_t i, int full, double rcu, int64_t* cnt) {
  *cnt = 0;
  const double* xi = &s->pos[3 * i];
  const int64_t mx = cm->maxneighbors;
  for (int64_t jp = 0; jp < cm->nv[i]; ++jp) {
    int64_t j = cm->vlist[i * mx + jp];
    if (!full && j < i)
      continue;
    double rij[3];
    orc_displacement(s->L, xi, &s->pos[3 * j], rij);
    double r2 = sqmod(rij);
    if (r2 < rcu * rcu) {
      int e = push_pair(s, cnt, j, rij, r2);
      if (e)
        return e;
    }
  }
  return ORC_OK;
}

/* LCBinary automatic grid, plugins/lcbinary.cc:52-107: sub-cells near cutoff/5, count made even. */
static int lcb_auto_n(double len, double cutoff) {
  double fnn = cutoff / 5.0;
  int n = 1;
  while (1) {
    double previo = fabs(len / n - fnn);
    n++;
    double actual = fabs(len / n - fnn);
    if (actual < 1E-3)
      break;
    else if (actual > previo) {
      n--;
      break;
    }
  }
  if ((n % 2) != 0)
    n++;
  return n;
}

/* The sub-cell of a position (cell.Fractional, floor, wrap above only), plugins/lcbinary.cc:163-178. */
static int64_t lcb_cell(const orc_cm* cm, const double L[3], const double* x) {
  int i = (int)floor(cm->nx * (x[0] / L[0]));
  int j = (int)floor(cm->ny * (x[1] / L[1]));
  int k = (int)floor(cm->nz * (x[2] / L[2]));
  if (i > cm->nx - 1)
    i -= cm->nx;
  if (j > cm->ny - 1)
    j -= cm->ny;
  if (k > cm->nz - 1)
    k -= cm->nz;
  return (int64_t)k * (cm->nx * cm->ny) + (int64_t)j * cm->nx + i;
}

/* LCBinary::UpdateCell, plugins/lcbinary.cc:50-193: grid (automatic once), sub-cell stencil of
 * half-width ceil(cutoff/d - 0.5) with one wrap per axis, one atom per sub-cell (the last one
 * binned); a shared sub-cell grows every count by 2 and starts over. */
static int lcb_update_cell(orc_sim* s, orc_cm* cm) {
  for (int round = 0; round < 1000; ++round) {
    if (cm->mode_auto) {
      cm->nx = lcb_auto_n(s->L[0], cm->cutoff);
      cm->ny = lcb_auto_n(s->L[1], cm->cutoff);
      cm->nz = lcb_auto_n(s->L[2], cm->cutoff);
      cm->mode_auto = 0;
    }
    const int nx = cm->nx, ny = cm->ny, nz = cm->nz;
    if (nx <= 0 || ny <= 0 || nz <= 0)
      return ORC_ERR_INVALID;
    const int64_t ncell = (int64_t)nx * ny * nz;
    if (cm->subcell == NULL) {
      double d = s->L[0] / (double)nx;
      if (s->L[1] / (double)ny < d)
        d = s->L[1] / (double)ny;
      if (s->L[2] / (double)nz < d)
        d = s->L[2] / (double)nz;
      int side = (int)ceil((cm->cutoff / d) - 0.5);
      cm->side = side;
      cm->cells_inside = (2 * side + 1) * (2 * side + 1) * (2 * side + 1);
      cm->subcell = (int*)malloc(sizeof(int) * (size_t)(ncell * cm->cells_inside));
      if (!cm->subcell)
        return ORC_ERR_NOMEM;
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) {
            int r = 0;
            int64_t q = (int64_t)k * (nx * ny) + j * nx + i;
            for (int dz = -side; dz <= side; ++dz)
              for (int dy = -side; dy <= side; ++dy)
                for (int dx = -side; dx <= side; ++dx) {
                  int z0 = i + dx, z1 = j + dy, z2 = k + dz;
                  if (z0 < 0)
                    z0 += nx;
                  else if (z0 > nx - 1)
                    z0 -= nx;
                  if (z1 < 0)
                    z1 += ny;
                  else if (z1 > ny - 1)
                    z1 -= ny;
                  if (z2 < 0)
                    z2 += nz;
                  else if (z2 > nz - 1)
                    z2 -= nz;
                  if (z0 < 0 || z0 >= nx || z1 < 0 || z1 >= ny || z2 < 0 || z2 >= nz)
                    return ORC_ERR_INVALID; /* a stencil wider than the grid: out of the reference's range */
                  cm->subcell[q * cm->cells_inside + (r++)] = z2 * (nx * ny) + z1 * nx + z0;
                }
          }
    }
    if (cm->binlist == NULL) {
      cm->binlist = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncell);
      if (!cm->binlist)
        return ORC_ERR_NOMEM;
    }
    for (int64_t c = 0; c < ncell; ++c)
      cm->binlist[c] = -1;
    int update = 0;
    for (int64_t r = 0; r < s->n; ++r) {
      int64_t q = lcb_cell(cm, s->L, &s->pos[3 * r]);
      if (q < 0 || q >= ncell)
        return ORC_ERR_INVALID;
      if (cm->binlist[q] != -1)
        update = 1;
      cm->binlist[q] = r;
    }
    if (!update)
      return ORC_OK;
    cm->nx += 2;
    cm->ny += 2;
    cm->nz += 2;
    free(cm->subcell);
    cm->subcell = NULL;
    free(cm->binlist);
    cm->binlist = NULL;
  }
  return ORC_ERR_INVALID;
}

/* LCBinary::BuildNeighborList, plugins/lcbinary.cc:216-254: the stencil's atoms, lower indices
 * only for a half list. */
static int lcb_list(orc_sim* s, orc_cm* cm, int64_t i, int full, double rcut, int64_t* cnt) {
  *cnt = 0;
  const double* xi = &s->pos[3 * i];
  const int* c = &cm->subcell[lcb_cell(cm, s->L, xi) * cm->cells_inside];
  for (int q = 0; q < cm->cells_inside; ++q) {
    int64_t z = cm->binlist[c[q]];
    if ((z < 0) || (z == i))
      continue;
    if ((z > i) && (full == 0))
      continue;
    double rij[3];
    orc_displacement(s->L, xi, &s->pos[3 * z], rij);
    double r2 = sqmod(rij);
    if (r2 < rcut * rcut) {
      int e = push_pair(s, cnt, z, rij, r2);
      if (e)
        return e;
    }
  }
  return ORC_OK;
}

/* MinimumImageCellManager, plugins/minimumimage.cc:55-100. */
static int mi_update_cell(orc_sim* s, orc_cm* cm) {
  if (fabs(cm->cutoff) < 1E-10) {
    for (int q = 0; q < 3; ++q)
      if (0.5 * s->L[q] > cm->cutoff)
        cm->cutoff = 0.5 * s->L[q];
  }
  return ORC_OK;
}

static int mi_list(orc_sim* s, int64_t i, int full, double rcu, int64_t* cnt) {
  *cnt = 0;
  if (rcu < 1.0E-10)
    return ORC_ERR_INVALID;
  const double* xi = &s->pos[3 * i];
  for (int64_t j = full ? 0 : i + 1; j < s->n; ++j) {
    if (j == i)
      continue;
    double rij[3];
    orc_displacement(s->L, xi, &s->pos[3 * j], rij);
    double r2 = sqmod(rij);
    if (r2 < rcu * rcu) {
      int e = push_pair(s, cnt, j, rij, r2);
      if (e)
        return e;
    }
  }
  return ORC_OK;
}

static int cm_update_cell(orc_sim* s) {
  orc_cm* cm = s->cm;
  if (!cm)
    return ORC_ERR_MISSING;
  s->update_cell_calls++;
  switch (cm->kind) {
  case ORC_CM_LINKEDCELL:
    return lc_update_cell(s, cm);
  case ORC_CM_VERLETLIST:
    return vl_update_cell(s, cm);
  case ORC_CM_MINIMUMIMAGE:
    return mi_update_cell(s, cm);
  case ORC_CM_LCBINARY:
    return lcb_update_cell(s, cm);
  }
  return ORC_ERR_INVALID;
}

static int cm_list(orc_sim* s, int64_t i, int full, double rcut, int64_t* cnt) {
  orc_cm* cm = s->cm;
  switch (cm->kind) {
  case ORC_CM_LINKEDCELL:
    return lc_list(s, cm, i, full, rcut, cnt);
  case ORC_CM_VERLETLIST:
    return vl_list(s, cm, i, full, rcut, cnt);
  case ORC_CM_MINIMUMIMAGE:
    return mi_list(s, i, full, rcut, cnt);
  case ORC_CM_LCBINARY:
    return lcb_list(s, cm, i, full, rcut, cnt);
  }
  return ORC_ERR_INVALID;
}

/* ------------------------------------------------------------------------------------------- */
/* Potentials                                                                                  */
/* ------------------------------------------------------------------------------------------- */

/* Potential::AppliesTo, liblpmd/simulation/potential.cc:23-27. */
static inline int applies_to(const orc_pot* p, int s1, int s2) {
  return ((p->spc_sum < 0) || ((s1 + s2) == p->spc_sum));
}

/* LennardJones::pairEnergy, plugins/lennardjones.cc:53-58. */
static double lj_energy(const orc_pot* p, double r) {
  const double sigma = p->p[0], epsilon = p->p[1];
  double rtmp = sigma / r;
  double r6 = rtmp * rtmp * rtmp * rtmp * rtmp * rtmp;
  double r12 = r6 * r6;
  return 4.0e0 * epsilon * (r12 - r6);
}

/* FastLJ::Tabulate, plugins/fastlj.cc:38-54: LJ at the lower edge of every bin. */
static int fastlj_tabulate(orc_pot* p) {
  const double sigma = p->p[0], epsilon = p->p[1], cutoff = p->p[2];
  p->tab = (double*)malloc(sizeof(double) * 2 * (size_t)p->bins);
  if (!p->tab)
    return ORC_ERR_NOMEM;
  for (long i = 0; i < p->bins; ++i) {
    double r = cutoff * (double)i / (double)p->bins;
    double r6 = pow(sigma / r, 6.0e0);
    double r12 = r6 * r6;
    p->tab[i] = 4.0e0 * epsilon * (r12 - r6);
    p->tab[p->bins + i] = -48.0e0 * (epsilon / (r * r)) * (r12 - 0.50e0 * r6);
  }
  return ORC_OK;
}

/* FastLJ::pairEnergy / pairForce, plugins/fastlj.cc:56-73: the bin floor(bins r / cutoff). */
static long fastlj_bin(const orc_pot* p, double r) { return (long)floor(p->bins * r / p->cutoff); }

static double fastlj_energy(const orc_pot* p, double r) { return p->tab[fastlj_bin(p, r)]; }

static void fastlj_force(const orc_pot* p, const double r[3], double out[3]) {
  double rr = sqrt(sqmod(r));
  double ff = p->tab[p->bins + fastlj_bin(p, rr)];
  out[0] = r[0] * ff;
  out[1] = r[1] * ff;
  out[2] = r[2] * ff;
}

/* LennardJones::pairForce, plugins/lennardjones.cc:60-67. */
static void lj_force(const orc_pot* p, const double r[3], double out[3]) {
  const double sigma = p->p[0], epsilon = p->p[1];
  double rr2 = sqmod(r);
  double r6 = pow(sigma * sigma / rr2, 3.0e0);
  double r12 = r6 * r6;
  double ff = -48.0e0 * (epsilon / rr2) * (r12 - 0.50e0 * r6);
  out[0] = r[0] * ff;
  out[1] = r[1] * ff;
  out[2] = r[2] * ff;
}

/* Metal functionals.  Sutton-Chen: plugins/suttonchen.cc:73-95; params {e,a,n,m,c,cutoff}.
 * Finnis-Sinclair: plugins/finnissinclair.cc:75-113; params {c0,c1,c2,A,B,c,d}.
 * Finnis-Sinclair-ext: plugins/finnissinclair-ext.cc:85-128; {c0,c1,c2,c3,c4,A,B,c,d}.
 * Gupta: plugins/gupta.cc:52-75; params {A,r0,p,B,q,cutoff}. */
static double metal_pair_energy(const orc_pot* p, double r) {
  if (p->kind == ORC_POT_GUPTA) {
    const double A = p->p[0], r0 = p->p[1], pp = p->p[2];
    return A * exp(-pp * (r - r0) / r0);
  }
  if (p->kind == ORC_POT_SC) {
    const double e = p->p[0], n = p->p[2];
    double ir = 1 / r;
    return e * p->an * pow(ir, n);
  } else if (p->kind == ORC_POT_FS) {
    const double c0 = p->p[0], c1 = p->p[1], c2 = p->p[2], c = p->p[5];
    if (r <= c)
      return (r - c) * (r - c) * (c0 + c1 * r + c2 * r * r);
    return 0.0e0;
  } else {
    const double c0 = p->p[0], c1 = p->p[1], c2 = p->p[2], c3 = p->p[3], c4 = p->p[4];
    const double c = p->p[7];
    if (r <= c) {
      double r2 = r * r;
      return (r - c) * (r - c) * (c0 + c1 * r + c2 * r2 + c3 * r2 * r + c4 * r2 * r2);
    }
    return 0.0e0;
  }
}

static double metal_rhoij(const orc_pot* p, double r) {
  if (p->kind == ORC_POT_GUPTA) {
    const double r0 = p->p[1], q = p->p[4];
    return exp(-2.0e0 * q * (r - r0) / r0);
  }
  if (p->kind == ORC_POT_SC) {
    const double m = p->p[3];
    double ir = 1 / r;
    return p->am * pow(ir, m);
  } else if (p->kind == ORC_POT_FS) {
    const double B = p->p[4], d = p->p[6];
    if (r <= d)
      return ((r - d) * (r - d)) * (1.0e0 + B * (r - d) / d);
    return 0.0e0;
  } else {
    const double B = p->p[6], d = p->p[8];
    if (r <= d) {
      double rd = r - d;
      return (rd * rd) * (1.0e0 + B * B * rd * rd);
    }
    return 0.0e0;
  }
}

static double metal_F(const orc_pot* p, double rhoi) {
  if (p->kind == ORC_POT_GUPTA)
    return -p->p[3] * sqrt(rhoi);
  if (p->kind == ORC_POT_SC) {
    const double e = p->p[0], c = p->p[4];
    return -c * e * sqrt(rhoi);
  } else if (p->kind == ORC_POT_FS) {
    return -p->p[3] * sqrt(rhoi);
  } else {
    return -p->p[5] * sqrt(rhoi);
  }
}

/* PairForce(normrij, r): a scalar times normrij; the scalar is returned. */
static double metal_pair_force(const orc_pot* p, double rmod) {
  if (p->kind == ORC_POT_GUPTA) {
    const double A = p->p[0], r0 = p->p[1], pp = p->p[2];
    return -(A * pp / r0) * exp(-pp * (rmod - r0) / r0);
  }
  if (p->kind == ORC_POT_SC) {
    const double e = p->p[0], n = p->p[2];
    double ir = 1.0e0 / rmod;
    return -n * e * p->an * pow(ir, n + 1);
  } else if (p->kind == ORC_POT_FS) {
    const double c0 = p->p[0], c1 = p->p[1], c2 = p->p[2], c = p->p[5];
    double r = rmod;
    if (r <= c) {
      double t1 = 2.0e0 * (r - c) * (c0 + c1 * r + c2 * r * r);
      double t2 = (r - c) * (r - c) * (c1 + 2.0e0 * c2 * r);
      return (t1 + t2);
    }
    return 0.0;
  } else {
    const double c0 = p->p[0], c1 = p->p[1], c2 = p->p[2], c3 = p->p[3], c4 = p->p[4];
    const double c = p->p[7];
    double r = rmod;
    if (r <= c) {
      double r2 = r * r;
      double rc = r - c;
      double t1 = 2.0e0 * rc * (c0 + c1 * r + c2 * r2 + c3 * r2 * r + c4 * r2 * r2);
      double t2 = (c1 + 2.0e0 * c2 * r + 3.0e0 * c3 * r2 + 4.0e0 * c4 * r2 * r) * rc * rc;
      return (t1 + t2);
    }
    return 0.0;
  }
}

/* ManyBodies(normrij, rhoi, rhoj, r): a scalar times normrij; the scalar is returned.
 * has_value tells whether the reference returns tmp*normrij (1) or Vector(0,0,0) (0); the
 * two differ only for -0.0 components, which do not change any sum. */
static double metal_many_bodies(const orc_pot* p, double rhoi, double rhoj, double rmod) {
  if (p->kind == ORC_POT_GUPTA) {
    const double r0 = p->p[1], B = p->p[3], q = p->p[4];
    return (B * q / r0) * ((1.0e0 / sqrt(rhoi)) + (1.0e0 / sqrt(rhoj))) * exp(-2.0e0 * q * (rmod - r0) / r0);
  }
  if (p->kind == ORC_POT_SC) {
    const double e = p->p[0], m = p->p[3], c = p->p[4];
    double ir = 1.0e0 / rmod;
    double tmp = 0.5 * m * c * e * ((1 / sqrt(rhoi)) + 1 / (sqrt(rhoj))) * p->am * pow(ir, m + 1);
    return tmp;
  } else if (p->kind == ORC_POT_FS) {
    const double A = p->p[3], B = p->p[4], d = p->p[6];
    double r = rmod;
    if (r <= d) {
      double t1 = ((1.0e0 / sqrt(rhoi)) + (1.0e0 / sqrt(rhoj))) * A / 2.0e0;
      double t2 = 2.0e0 * (r - d) + 3.0e0 * B * (r - d) * (r - d) / d;
      return -t1 * t2;
    }
    return 0.0;
  } else {
    const double A = p->p[5], B = p->p[6], d = p->p[8];
    double r = rmod;
    if (r <= d) {
      double rd = r - d;
      double t1 = A * 0.5e0 * ((1.0e0 / sqrt(rhoi)) + (1.0e0 / sqrt(rhoj)));
      double t2 = 2.0e0 * rd + 4.0e0 * B * B * rd * rd * rd;
      return -t1 * t2;
    }
    return 0.0;
  }
}

/* PairPotential::UpdateForces, liblpmd/simulation/pairpotential.cc:35-84. */
static int pair_update_forces(orc_sim* s, int pi) {
  orc_pot* p = &s->pots[pi];
  const double forcefactor = ORC_FORCEFACTOR;
  const int64_t n = s->n;
  double stress[3][3];
  double etmp = 0.0e0, tmpvir = 0.0e0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      stress[i][j] = 0.0e0;
  const double cutoff = p->cutoff;
  for (int64_t i = 0; i < n; ++i) {
    int64_t cnt;
    int e = cm_list(s, i, 0, cutoff, &cnt);
    if (e)
      return e;
    for (int64_t k = 0; k < cnt; ++k) {
      int64_t j = s->lj[k];
      const double* rij = &s->lrij[3 * k];
      double r2 = s->lr2[k];
      if (applies_to(p, s->Z[i], s->Z[j]) && r2 < cutoff * cutoff) {
        double ff[3];
        if (p->kind == ORC_POT_FASTLJ) {
          etmp += fastlj_energy(p, sqrt(r2));
          fastlj_force(p, rij, ff);
        } else {
          etmp += lj_energy(p, sqrt(r2));
          lj_force(p, rij, ff);
        }
        double fi = (forcefactor / s->mass[i]);
        double fj = (forcefactor / s->mass[j]);
        for (int q = 0; q < 3; ++q)
          s->acc[3 * i + q] += ff[q] * fi;
        for (int q = 0; q < 3; ++q)
          s->acc[3 * j + q] -= ff[q] * fj;
        tmpvir -= (rij[0] * ff[0] + rij[1] * ff[1] + rij[2] * ff[2]);
        for (int l = 0; l < 3; ++l) {
          stress[0][l] += -(rij)[0] * ff[l];
          stress[1][l] += -(rij)[1] * ff[l];
          stress[2][l] += -(rij)[2] * ff[l];
        }
      }
    }
  }
  s->energy[pi] = 0.0 + etmp;
  s->virial += tmpvir;
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      s->stress[b][a] = s->stress[b][a] + stress[b][a];
  return ORC_OK;
}

/* MetalPotential::UpdateForces, liblpmd/simulation/metalpotential.cc:62-180.
 * The first-call correction pass (:86-116) only prints diagnostics (du, dvir and the mean
 * particle density stay 0), so it is not restated.  The reference leaves its local stress
 * accumulator uninitialised (:68); it is zeroed here. */
static int metal_update_forces(orc_sim* s, int pi) {
  orc_pot* p = &s->pots[pi];
  const double forcefactor = ORC_FORCEFACTOR;
  const int64_t n = s->n;
  double stress[3][3];
  double tmpvir = 0.0e0, etmp = 0.0e0, etmp2 = 0.0e0;
  const double mpd = 0.0;
  const double du = 0.0e0, dvir = 0.0e0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      stress[i][j] = 0.0e0;
  free(p->rho);
  p->rho = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  if (!p->rho)
    return ORC_ERR_NOMEM;
  for (int64_t i = 0; i < n; ++i)
    p->rho[i] = 0.0e0;
  const double rc = p->cutoff;
  for (int64_t i = 0; i < n; ++i) {
    double rhoi = 0.0e0;
    int64_t cnt;
    int e = cm_list(s, i, 1, rc, &cnt);
    if (e)
      return e;
    for (int64_t k = 0; k < cnt; ++k)
      rhoi += metal_rhoij(p, sqrt(s->lr2[k]));
    p->rho[i] = rhoi + mpd;
  }
  for (int64_t i = 0; i < n; ++i) {
    int64_t cnt;
    int e = cm_list(s, i, 0, rc, &cnt);
    if (e)
      return e;
    for (int64_t k = 0; k < cnt; ++k) {
      int64_t j = s->lj[k];
      const double* rij = &s->lrij[3 * k];
      if (applies_to(p, s->Z[i], s->Z[j])) {
        double r = sqrt(s->lr2[k]);
        double norm[3] = {rij[0], rij[1], rij[2]};
        double mod = sqrt(norm[0] * norm[0] + norm[1] * norm[1] + norm[2] * norm[2]);
        for (int q = 0; q < 3; ++q)
          norm[q] /= mod;
        etmp += metal_pair_energy(p, r);
        double pfs = metal_pair_force(p, r);
        double mbs = metal_many_bodies(p, p->rho[i], p->rho[j], r);
        double f[3];
        for (int q = 0; q < 3; ++q)
          f[q] = pfs * norm[q] + mbs * norm[q];
        double fi = (forcefactor / s->mass[i]);
        double fj = (forcefactor / s->mass[j]);
        for (int q = 0; q < 3; ++q)
          s->acc[3 * i + q] += f[q] * fi;
        for (int q = 0; q < 3; ++q)
          s->acc[3 * j + q] -= f[q] * fj;
        tmpvir -= (rij[0] * f[0] + rij[1] * f[1] + rij[2] * f[2]);
        for (int q = 0; q < 3; q++) {
          stress[0][q] += -(rij)[0] * f[q];
          stress[1][q] += -(rij)[1] * f[q];
          stress[2][q] += -(rij)[2] * f[q];
        }
      }
    }
    etmp2 += metal_F(p, p->rho[i]);
  }
  s->energy[pi] = 0.0 + (etmp + du + etmp2);
  s->virial += tmpvir + dvir;
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      s->stress[b][a] = s->stress[b][a] + stress[b][a];
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------------- */
/* Simulation                                                                                  */
/* ------------------------------------------------------------------------------------------- */

orc_sim* orc_sim_create(int64_t n, const double L[3]) {
  if (n < 0)
    return NULL;
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  if (!s)
    return NULL;
  s->n = n;
  for (int q = 0; q < 3; ++q)
    s->L[q] = L[q];
  size_t m = (size_t)(n > 0 ? n : 1);
  s->pos = (double*)calloc(3 * m, sizeof(double));
  s->vel = (double*)calloc(3 * m, sizeof(double));
  s->acc = (double*)calloc(3 * m, sizeof(double));
  s->old_acc = (double*)calloc(3 * m, sizeof(double));
  s->Z = (int32_t*)calloc(m, sizeof(int32_t));
  s->mass = (double*)calloc(m, sizeof(double));
  s->flags = (uint8_t*)calloc(m, 1);
  if (!s->pos || !s->vel || !s->acc || !s->old_acc || !s->Z || !s->mass || !s->flags) {
    orc_sim_destroy(s);
    return NULL;
  }
  if (ensure_scratch(s, 256)) {
    orc_sim_destroy(s);
    return NULL;
  }
  return s;
}

void orc_sim_destroy(orc_sim* s) {
  if (!s)
    return;
  free(s->pos);
  free(s->vel);
  free(s->acc);
  free(s->old_acc);
  free(s->old_pos);
  free(s->old_vel);
  free(s->aux);
  free(s->Z);
  free(s->mass);
  free(s->flags);
  for (int i = 0; i < s->npots; ++i) {
    free(s->pots[i].rho);
    free(s->pots[i].tab);
  }
  cm_free(s->cm);
  free(s->lj);
  free(s->lrij);
  free(s->lr2);
  free(s);
}

int orc_sim_set_atoms(orc_sim* s, const double* pos, const double* vel, const double* acc,
                      const int32_t* Z, const double* mass) {
  size_t m = (size_t)s->n;
  if (pos)
    memcpy(s->pos, pos, 3 * m * sizeof(double));
  if (vel)
    memcpy(s->vel, vel, 3 * m * sizeof(double));
  else
    memset(s->vel, 0, 3 * m * sizeof(double));
  if (acc)
    memcpy(s->acc, acc, 3 * m * sizeof(double));
  else
    memset(s->acc, 0, 3 * m * sizeof(double));
  if (Z)
    memcpy(s->Z, Z, m * sizeof(int32_t));
  if (mass)
    memcpy(s->mass, mass, m * sizeof(double));
  return ORC_OK;
}

int orc_sim_set_flags(orc_sim* s, const uint8_t* flags) {
  s->have_fixedvel = s->have_fixedpos = 0;
  for (int64_t i = 0; i < s->n; ++i) {
    s->flags[i] = flags ? flags[i] : 0;
    if (s->flags[i] & ORC_FIXEDVEL)
      s->have_fixedvel = 1;
    if (s->flags[i] & ORC_FIXEDPOS)
      s->have_fixedpos = 1;
  }
  return ORC_OK;
}

int orc_sim_get_atoms(const orc_sim* s, double* pos, double* vel, double* acc) {
  size_t m = (size_t)s->n;
  if (pos)
    memcpy(pos, s->pos, 3 * m * sizeof(double));
  if (vel)
    memcpy(vel, s->vel, 3 * m * sizeof(double));
  if (acc)
    memcpy(acc, s->acc, 3 * m * sizeof(double));
  return ORC_OK;
}

static int set_cm(orc_sim* s, orc_cm* cm) {
  cm_free(s->cm);
  s->cm = cm;
  return cm_update_cell(s); /* Configuration::SetCellManager calls UpdateCell */
}

int orc_sim_set_linkedcell(orc_sim* s, double cutoff, int nx, int ny, int nz, int mode_auto) {
  orc_cm* cm = (orc_cm*)calloc(1, sizeof(orc_cm));
  if (!cm)
    return ORC_ERR_NOMEM;
  cm->kind = ORC_CM_LINKEDCELL;
  cm->cutoff = cutoff;
  cm->nx = nx;
  cm->ny = ny;
  cm->nz = nz;
  cm->mode_auto = mode_auto;
  cm->last_atoms_size = -1;
  return set_cm(s, cm);
}

int orc_sim_set_verletlist(orc_sim* s, double cutoff, int64_t maxneighbors, int64_t each) {
  if (each <= 0 || maxneighbors <= 1)
    return ORC_ERR_INVALID;
  orc_cm* cm = (orc_cm*)calloc(1, sizeof(orc_cm));
  if (!cm)
    return ORC_ERR_NOMEM;
  cm->kind = ORC_CM_VERLETLIST;
  cm->cutoff = cutoff;
  cm->maxneighbors = maxneighbors;
  cm->each = each;
  /* verletlist.cc:24-25: extcut is never read from "extcutoff"; it ends up 1.08*cutoff. */
  cm->extcut = 1.08 * cutoff;
  cm->step_count = 0;
  cm->old_size = 0;
  return set_cm(s, cm);
}

int orc_sim_set_lcbinary(orc_sim* s, double cutoff, int nx, int ny, int nz, int mode_auto) {
  orc_cm* cm = (orc_cm*)calloc(1, sizeof(orc_cm));
  if (!cm)
    return ORC_ERR_NOMEM;
  cm->kind = ORC_CM_LCBINARY;
  cm->cutoff = cutoff;
  cm->nx = nx;
  cm->ny = ny;
  cm->nz = nz;
  /* plugins/lcbinary.cc:23-28: a zero count or mode auto selects the automatic grid */
  cm->mode_auto = mode_auto || nx == 0 || ny == 0 || nz == 0;
  return set_cm(s, cm);
}

int orc_sim_set_minimumimage(orc_sim* s, double cutoff) {
  orc_cm* cm = (orc_cm*)calloc(1, sizeof(orc_cm));
  if (!cm)
    return ORC_ERR_NOMEM;
  cm->kind = ORC_CM_MINIMUMIMAGE;
  cm->cutoff = cutoff;
  return set_cm(s, cm);
}

int orc_sim_add_potential(orc_sim* s, int kind, const double* params, int nparams, int s1, int s2) {
  if (s->npots >= ORC_MAXPOT)
    return ORC_ERR_INVALID;
  int need = (kind == ORC_POT_LJ) ? 3 : (kind == ORC_POT_FASTLJ) ? 4
           : (kind == ORC_POT_SC || kind == ORC_POT_GUPTA) ? 6 : (kind == ORC_POT_FS) ? 7 : 9;
  if (kind < ORC_POT_LJ || kind > ORC_POT_FASTLJ || nparams < need)
    return ORC_ERR_INVALID;
  orc_pot* p = &s->pots[s->npots];
  memset(p, 0, sizeof(*p));
  p->kind = kind;
  for (int i = 0; i < need; ++i)
    p->p[i] = params[i];
  p->spc_sum = s1 + s2;
  if (kind == ORC_POT_LJ) {
    p->cutoff = params[2];
  } else if (kind == ORC_POT_SC) {
    p->cutoff = params[5];
    p->an = pow(params[1], params[2]); /* suttonchen.cc:29-30 */
    p->am = pow(params[1], params[3]);
  } else if (kind == ORC_POT_GUPTA) {
    p->cutoff = params[5]; /* gupta.cc:26 */
  } else if (kind == ORC_POT_FASTLJ) {
    p->cutoff = params[2]; /* fastlj.cc:24 */
    p->bins = (long)params[3];
    if (p->bins < 1)
      return ORC_ERR_INVALID;
    if (fastlj_tabulate(p) != ORC_OK)
      return ORC_ERR_NOMEM;
  } else if (kind == ORC_POT_FS) {
    double c = params[5], d = params[6];
    p->cutoff = (d >= c) ? d : c; /* finnissinclair.cc:27-30 */
  } else {
    double c = params[7], d = params[8];
    p->cutoff = (d >= c) ? d : c;
  }
  s->npots++;
  return ORC_OK;
}

int orc_sim_set_velocityverlet(orc_sim* s, double dt) { return orc_sim_set_integrator(s, ORC_INT_VV, dt, 0.0, 300.0); }

int orc_sim_set_integrator(orc_sim* s, int kind, double dt, double fmass, double t) {
  if (kind < ORC_INT_VV || kind > ORC_INT_NOSEHOOVER)
    return ORC_ERR_INVALID;
  if (kind == ORC_INT_NOSEHOOVER && !(fmass > 0.0))
    return ORC_ERR_INVALID;
  s->integ = kind;
  s->dt = dt;
  s->fmass = fmass;
  s->t0 = t;
  s->have_integrator = 1;
  return ORC_OK;
}

/* CombinedPotential::UpdateForces, liblpmd/lpmd/combinedpotential.h:39-52. */
int orc_sim_update_forces(orc_sim* s) {
  for (int64_t i = 0; i < 3 * s->n; ++i)
    s->acc[i] = 0.0;
  s->virial = 0.0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      s->stress[a][b] = 0.0;
  int e = cm_update_cell(s);
  if (e)
    return e;
  for (int p = 0; p < s->npots; ++p) {
    e = (s->pots[p].kind == ORC_POT_LJ || s->pots[p].kind == ORC_POT_FASTLJ) ? pair_update_forces(s, p)
                                                                             : metal_update_forces(s, p);
    if (e)
      return e;
  }
  return ORC_OK;
}

double orc_sim_energy(const orc_sim* s) {
  double en = 0.0;
  for (int p = 0; p < s->npots; ++p)
    en += s->energy[p];
  return en;
}

double orc_sim_virial(const orc_sim* s) { return s->virial; }

void orc_sim_stress(const orc_sim* s, double out[9]) {
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      out[3 * a + b] = s->stress[a][b];
}

/* VelocityVerlet::AdvancePosition, plugins/velocityverlet.cc:60-68. */
static void vv_advance_position(orc_sim* s, int64_t i) {
  const double dt = s->dt;
  double* x = &s->pos[3 * i];
  const double* v = &s->vel[3 * i];
  const double* a = &s->acc[3 * i];
  double np[3];
  for (int q = 0; q < 3; ++q)
    np[q] = x[q] + v[q] * dt + 0.5 * a[q] * dt * dt;
  for (int q = 0; q < 3; ++q)
    s->old_acc[3 * i + q] = a[q];
  orc_fitted_inside(s->L, np, x);
}

/* VelocityVerlet::AdvanceVelocity, plugins/velocityverlet.cc:70-75. */
static void vv_advance_velocity(orc_sim* s, int64_t i) {
  const double dt = s->dt;
  double* v = &s->vel[3 * i];
  for (int q = 0; q < 3; ++q)
    v[q] = v[q] + 0.5 * dt * (s->old_acc[3 * i + q] + s->acc[3 * i + q]);
}

static void zero_fixedvel(orc_sim* s) {
  if (!s->have_fixedvel)
    return;
  for (int64_t i = 0; i < s->n; ++i)
    if (s->flags[i] & ORC_FIXEDVEL)
      s->acc[3 * i] = s->acc[3 * i + 1] = s->acc[3 * i + 2] = 0.0;
}

/* TwoStepIntegrator::Advance, liblpmd/simulation/twostepintegrator.cc:12-68. */
static int vv_advance(orc_sim* s) {
  int e = orc_sim_update_forces(s);
  if (e)
    return e;
  zero_fixedvel(s);
  for (int64_t i = 0; i < s->n; ++i)
    if (!(s->have_fixedpos && (s->flags[i] & ORC_FIXEDPOS)))
      vv_advance_position(s, i);
  e = orc_sim_update_forces(s);
  if (e)
    return e;
  zero_fixedvel(s);
  for (int64_t i = 0; i < s->n; ++i)
    if (!(s->have_fixedpos && (s->flags[i] & ORC_FIXEDPOS)))
      vv_advance_velocity(s, i);
  return ORC_OK;
}

/* ---- the integrators other than velocityverlet ------------------------------------------ */

/* Integrator::GoBack on the backed-up copy, liblpmd/simulation/integrator.cc:31-42:
 * positions Fit(x - v dt), velocities v - a dt. */
static int go_back(orc_sim* s) {
  const size_t b = sizeof(double) * 3 * (size_t)(s->n > 0 ? s->n : 1);
  if (!s->old_pos)
    s->old_pos = (double*)malloc(b);
  if (!s->old_vel)
    s->old_vel = (double*)malloc(b);
  if (!s->aux)
    s->aux = (double*)calloc(3 * (size_t)(s->n > 0 ? s->n : 1), sizeof(double));
  if (!s->old_pos || !s->old_vel || !s->aux)
    return ORC_ERR_NOMEM;
  const double dt = s->dt;
  for (int64_t i = 0; i < s->n; ++i) {
    double np[3];
    for (int q = 0; q < 3; ++q) {
      np[q] = s->pos[3 * i + q] - s->vel[3 * i + q] * dt;
      s->old_vel[3 * i + q] = s->vel[3 * i + q] - s->acc[3 * i + q] * dt;
    }
    orc_fitted_inside(s->L, np, &s->old_pos[3 * i]);
  }
  return ORC_OK;
}

/* Potential::UpdateForces on the backed-up configuration (its own accelerations, virial and
 * stress; the cell manager is the shared one): the accelerations land in out[3n]. */
static int old_config_forces(orc_sim* s, double* out) {
  const size_t b = sizeof(double) * 3 * (size_t)s->n;
  double* save_acc = (double*)malloc(b ? b : 1);
  if (!save_acc)
    return ORC_ERR_NOMEM;
  memcpy(save_acc, s->acc, b);
  double save_virial = s->virial, save_stress[3][3], save_energy[ORC_MAXPOT];
  memcpy(save_stress, s->stress, sizeof(save_stress));
  memcpy(save_energy, s->energy, sizeof(save_energy));
  double* cur = s->pos;
  s->pos = s->old_pos;
  int e = orc_sim_update_forces(s);
  s->pos = cur;
  if (e == ORC_OK)
    memcpy(out, s->acc, b);
  memcpy(s->acc, save_acc, b);
  s->virial = save_virial;
  memcpy(s->stress, save_stress, sizeof(save_stress));
  memcpy(s->energy, save_energy, sizeof(save_energy));
  free(save_acc);
  return e;
}

/* Initialize of each integrator (SimulationEngine::DoStep's first call):
 *   velocityverlet, verlet  UseOldConfig (one UpdateCell on the copy, then GoBack)
 *   euler                   nothing (Integrator::Initialize)
 *   leapfrog                UseOldConfig, UpdateForces(OldConfig), v_old += a_old 0.5 dt
 *                           (plugins/leapfrog.cc:36-45)
 *   beeman, nosehoover      UseOldConfig, UpdateForces(OldConfig); aux = 0, friction 0
 *                           (plugins/beeman.cc:37-43, plugins/nosehoover.cc:35-42) */
static int integ_initialize(orc_sim* s) {
  if (s->integ == ORC_INT_EULER)
    return ORC_OK;
  int e = cm_update_cell(s);
  if (e || s->integ == ORC_INT_VV)
    return e;
  if ((e = go_back(s)))
    return e;
  if (s->integ == ORC_INT_VERLET)
    return ORC_OK;
  double* a_old = (double*)malloc(sizeof(double) * 3 * (size_t)(s->n > 0 ? s->n : 1));
  if (!a_old)
    return ORC_ERR_NOMEM;
  e = old_config_forces(s, a_old);
  if (e == ORC_OK) {
    for (int64_t k = 0; k < 3 * s->n; ++k) {
      if (s->integ == ORC_INT_LEAPFROG) {
        s->old_vel[k] += a_old[k] * 0.5 * s->dt;
      } else {
        s->old_acc[k] = a_old[k];
        s->aux[k] = 0.0;
      }
    }
    s->friction = 0.0;
  }
  free(a_old);
  return e;
}

static int moves(const orc_sim* s, int64_t i) { return !(s->have_fixedpos && (s->flags[i] & ORC_FIXEDPOS)); }

/* Euler::Advance (plugins/euler.cc:37-43), Leapfrog::Advance (plugins/leapfrog.cc:47-57),
 * Verlet::Advance (plugins/verlet.cc:41-55); OneStepIntegrator::Advance around them
 * (liblpmd/simulation/onestepintegrator.cc:13-40). */
static int onestep_advance(orc_sim* s) {
  int e = orc_sim_update_forces(s);
  if (e)
    return e;
  zero_fixedvel(s);
  const double dt = s->dt;
  for (int64_t i = 0; i < s->n; ++i) {
    if (!moves(s, i))
      continue;
    double* x = &s->pos[3 * i];
    double* v = &s->vel[3 * i];
    const double* a = &s->acc[3 * i];
    double np[3];
    if (s->integ == ORC_INT_EULER) {
      for (int q = 0; q < 3; ++q)
        np[q] = x[q] + v[q] * dt;
      orc_fitted_inside(s->L, np, x);
      for (int q = 0; q < 3; ++q)
        v[q] += a[q] * dt;
    } else if (s->integ == ORC_INT_LEAPFROG) {
      double* ov = &s->old_vel[3 * i];
      double vh[3];
      for (int q = 0; q < 3; ++q) {
        vh[q] = ov[q] + a[q] * dt;
        np[q] = x[q] + vh[q] * dt;
      }
      orc_fitted_inside(s->L, np, x);
      for (int q = 0; q < 3; ++q) {
        v[q] = (vh[q] + ov[q]) * 0.5;
        ov[q] = vh[q];
      }
    } else { /* verlet */
      double* op = &s->old_pos[3 * i];
      double oldpos[3];
      for (int q = 0; q < 3; ++q) {
        oldpos[q] = op[q];
        np[q] = (x[q] * 2.0 - op[q]) + a[q] * dt * dt;
        op[q] = x[q];
        s->old_vel[3 * i + q] = v[q];
      }
      orc_fitted_inside(s->L, np, x);
      double d[3];
      orc_displacement(s->L, oldpos, x, d);
      for (int q = 0; q < 3; ++q)
        v[q] = d[q] / (2.0 * dt);
    }
  }
  return ORC_OK;
}

/* Beeman (plugins/beeman.cc:45-70) and NoseHoover (plugins/nosehoover.cc:44-83) under
 * TwoStepIntegrator::Advance.  Nose-Hoover adds its friction increment for every moving atom,
 * in atom order, before that atom's update; the temperature is that of all atoms (tag false),
 * the Boltzmann constant the session's 0.00008617 (liblpmd/runtime/session.cc:17-32). */
static int twostep_advance(orc_sim* s) {
  int e = orc_sim_update_forces(s);
  if (e)
    return e;
  zero_fixedvel(s);
  const double dt = s->dt;
  double inc = 0.0;
  if (s->integ == ORC_INT_NOSEHOOVER) {
    double K = 0.0;
    for (int64_t i = 0; i < s->n; ++i)
      K += 0.5 * s->mass[i] * sqmod(&s->vel[3 * i]);
    double T = (s->n == 0) ? 0.0 : (2.0 / 3.0) * (K * ORC_KIN2EV) / (ORC_KBOLTZMANN * (double)s->n);
    inc = ((3.0 * (double)s->n / s->fmass) * 0.00008617 * (T - s->t0) * dt);
  }
  for (int64_t i = 0; i < s->n; ++i) {
    if (!moves(s, i))
      continue;
    double* x = &s->pos[3 * i];
    const double* v = &s->vel[3 * i];
    double* a = &s->acc[3 * i];
    double* oa = &s->old_acc[3 * i];
    double na[3], np[3];
    if (s->integ == ORC_INT_NOSEHOOVER) {
      s->friction += inc;
      for (int q = 0; q < 3; ++q) {
        na[q] = a[q] - v[q] * s->friction;
        a[q] = na[q];
      }
    } else {
      for (int q = 0; q < 3; ++q)
        na[q] = a[q];
    }
    for (int q = 0; q < 3; ++q) {
      s->aux[3 * i + q] = oa[q];
      np[q] = x[q] + v[q] * dt + na[q] * (2.0 / 3.0) * dt * dt - oa[q] * (1.0 / 6.0) * dt * dt;
      oa[q] = na[q];
    }
    orc_fitted_inside(s->L, np, x);
  }
  e = orc_sim_update_forces(s);
  if (e)
    return e;
  zero_fixedvel(s);
  for (int64_t i = 0; i < s->n; ++i) {
    if (!moves(s, i))
      continue;
    double* v = &s->vel[3 * i];
    for (int q = 0; q < 3; ++q)
      v[q] = v[q] + s->acc[3 * i + q] * (1.0 / 3.0) * dt + s->old_acc[3 * i + q] * (5.0 / 6.0) * dt -
             s->aux[3 * i + q] * (1.0 / 6.0) * dt;
  }
  return ORC_OK;
}

/* KineticEnergy / Temperature / Momentum, liblpmd/lpmd/properties.h:22-81, and
 * SetSimulationTags, liblpmd/simulation/simulationbuilder.cc:84-124. */
int orc_sim_thermo(const orc_sim* s, double* out) {
  const int tag = s->have_fixedvel || s->have_fixedpos;
  double K = 0.0;
  double P[3] = {0.0, 0.0, 0.0};
  int64_t skipped = 0;
  for (int64_t i = 0; i < s->n; ++i) {
    if (tag && (s->flags[i] & (ORC_FIXEDVEL | ORC_FIXEDPOS))) {
      skipped++;
      continue;
    }
    const double* v = &s->vel[3 * i];
    K += 0.5 * s->mass[i] * sqmod(v);
    for (int q = 0; q < 3; ++q)
      P[q] += (v[q] * s->mass[i]);
  }
  double kin = K * ORC_KIN2EV;
  double temp = (s->n == 0) ? 0.0 : (2.0 / 3.0) * kin / (ORC_KBOLTZMANN * (double)(s->n - skipped));
  double vol = s->L[0] * s->L[1] * s->L[2];
  double epot = orc_sim_energy(s);
  memset(out, 0, sizeof(double) * ORC_THERMO_LEN);
  out[ORC_T_STEP] = (double)s->step;
  out[ORC_T_EPOT] = epot;
  out[ORC_T_EKIN] = kin;
  out[ORC_T_ETOT] = epot + kin;
  out[ORC_T_TEMP] = temp;
  out[ORC_T_VIRIAL] = s->virial;
  out[ORC_T_PX] = P[0];
  out[ORC_T_PY] = P[1];
  out[ORC_T_PZ] = P[2];
  out[ORC_T_VOLUME] = vol;
  out[ORC_T_VIRIAL_PRESSURE] = (ORC_PRESSFACTOR / vol) * (1.0 / 3.0) * s->virial;
  out[ORC_T_KINETIC_PRESSURE] = (ORC_PRESSFACTOR / vol) * (2.0 / 3.0) * kin;
  out[ORC_T_PRESSURE] = (ORC_PRESSFACTOR / vol) * ((2.0 / 3.0) * kin + (1.0 / 3.0) * s->virial);
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      out[ORC_T_STRESS + 3 * a + b] = s->stress[a][b];
  return ORC_OK;
}

/* SimulationEngine::DoStep, liblpmd/simulation/simulationbuilder.cc:126-136.  The first
 * call runs VelocityVerlet::Initialize -> Integrator::UseOldConfig, which attaches the cell
 * manager to a copy of the configuration and so makes one more UpdateCell call on the
 * current positions (liblpmd/simulation/integrator.cc:16-22). */
int orc_sim_do_steps(orc_sim* s, int64_t nsteps, double* thermo) {
  if (!s->have_integrator)
    return ORC_ERR_MISSING;
  if (!s->cm)
    return ORC_ERR_MISSING;
  for (int64_t k = 0; k < nsteps; ++k) {
    s->virial = 0.0;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        s->stress[a][b] = 0.0;
    if (!s->initialized) {
      int e = integ_initialize(s);
      if (e)
        return e;
      s->initialized = 1;
    }
    int e = (s->integ == ORC_INT_VV) ? vv_advance(s)
            : (s->integ == ORC_INT_BEEMAN || s->integ == ORC_INT_NOSEHOOVER) ? twostep_advance(s)
                                                                           : onestep_advance(s);
    if (e)
      return e;
    s->step++;
    if (thermo)
      orc_sim_thermo(s, thermo + k * ORC_THERMO_LEN);
  }
  return ORC_OK;
}

int orc_sim_neighbors(orc_sim* s, int full, double rcut, int64_t* counts, int64_t* idx,
                      int64_t cap, int64_t* total) {
  if (!s->cm)
    return ORC_ERR_MISSING;
  int64_t t = 0;
  int rc = ORC_OK;
  for (int64_t i = 0; i < s->n; ++i) {
    int64_t cnt;
    int e = cm_list(s, i, full, rcut, &cnt);
    if (e)
      return e;
    if (counts)
      counts[i] = cnt;
    for (int64_t k = 0; k < cnt; ++k) {
      if (idx && t < cap)
        idx[t] = s->lj[k];
      else if (idx)
        rc = ORC_ERR_CAPACITY;
      t++;
    }
  }
  if (total)
    *total = t;
  return rc;
}

int64_t orc_sim_update_cell_calls(const orc_sim* s) { return s->update_cell_calls; }
