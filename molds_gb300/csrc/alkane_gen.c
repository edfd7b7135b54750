/*
 * Random saturated acyclic alkanes C_n H_(2n+2) with ideal geometry (host
 * code; inputs of the uneven-batch and serving workloads).
 *
 * Topology: carbon k (k >= 1) attaches to a uniformly chosen earlier carbon
 * that has fewer than 4 carbon neighbours.  Geometry: C-C 1.54 A, C-H 1.09 A,
 * tetrahedral angles, root orientation uniformly random; carbons are placed
 * breadth first and each carbon's dihedral about the bond to its parent is
 * drawn uniformly in [0, 2 pi).  `attempts` draws are tested at once; the
 * first clash-free one is kept.  A clash is a pair of atoms >= 3 bonds apart
 * closer than min_cc (both carbons) or min_other (any other pair).  When no
 * draw is clash-free the search jumps back to the latest carbon that placed a
 * clashing atom (conflict-directed backjumping); after `budget` draws the
 * tree is redrawn.  Deterministic for a seed (xoshiro256** seeded by
 * splitmix64; plain double arithmetic).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { uint64_t s[4]; } rng_t;

static uint64_t splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t next_u64(rng_t* r) {
  uint64_t* s = r->s;
  const uint64_t out = rotl(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
  return out;
}

static double uniform01(rng_t* r) { return (double)(next_u64(r) >> 11) * (1.0 / 9007199254740992.0); }

static int uniform_int(rng_t* r, int k) { return (int)(uniform01(r) * k); }

static double normal01(rng_t* r) {
  double u1 = uniform01(r), u2 = uniform01(r);
  if (u1 < 1e-300) u1 = 1e-300;
  return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

static void sub3(const double* a, const double* b, double* o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; }
static void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
static void unit3(double* v) {
  const double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= n; v[1] /= n; v[2] /= n;
}

/* children of the root live in kids[0..3], those of carbon c >= 1 in kids[KB(c)..KB(c)+2] */
#define KB(c) ((c) == 0 ? 0 : 4 + 3 * ((c) - 1))

#define CC_BOND 1.54
#define CH_BOND 1.09

typedef struct {
  int n, total, count;
  int* parent;
  int* nkids;
  int* kids;        /* see KB() */
  int* order;
  int* idx_of_c;
  int* start_count;
  double* ref;      /* 3 per carbon: reference atom of the dihedral frame */
  int* Z;
  double* pos;      /* 3 per atom */
  int* owner;       /* order index of the carbon that placed an atom (-1: root) */
  unsigned short* D;/* bond-graph distances among placed atoms, total x total */
} grow_t;

static int add_atom(grow_t* g, int z, const double* p, int bonded_to, int t) {
  const int i = g->count;
  g->Z[i] = z;
  memcpy(g->pos + 3 * i, p, 3 * sizeof(double));
  g->owner[i] = t;
  if (bonded_to >= 0) {
    unsigned short* Di = g->D + (size_t)i * g->total;
    const unsigned short* Db = g->D + (size_t)bonded_to * g->total;
    for (int j = 0; j < i; ++j) {
      const unsigned short d = (unsigned short)(Db[j] + 1);
      Di[j] = d;
      g->D[(size_t)j * g->total + i] = d;
    }
  }
  g->D[(size_t)i * g->total + i] = 0;
  g->count++;
  return i;
}

/* returns 1 on success */
static int grow(grow_t* g, rng_t* r, double min_cc, double min_other, int attempts, long long budget) {
  const int n = g->n;
  const double tet = acos(-1.0 / 3.0);
  const double ct = cos(tet), st = sin(tet);
  /* breadth-first order of the non-root carbons */
  int head = 0, tail = 0;
  for (int k = 0; k < g->nkids[0]; ++k) g->order[tail++] = g->kids[k];
  while (head < tail) {
    const int c = g->order[head++];
    for (int k = 0; k < g->nkids[c]; ++k) g->order[tail++] = g->kids[KB(c) + k];
  }
  /* root: random orientation of a regular tetrahedron */
  double q[4];
  double qn = 0.0;
  for (int k = 0; k < 4; ++k) { q[k] = normal01(r); qn += q[k] * q[k]; }
  qn = sqrt(qn);
  for (int k = 0; k < 4; ++k) q[k] /= qn;
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)},
                          {2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)},
                          {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)}};
  const double base[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
  double tdir[4][3];
  for (int i = 0; i < 4; ++i)
    for (int a = 0; a < 3; ++a) {
      double s = 0.0;
      for (int b = 0; b < 3; ++b) s += R[a][b] * base[i][b] / sqrt(3.0);
      tdir[i][a] = s;
    }
  g->count = 0;
  const double zero[3] = {0, 0, 0};
  g->idx_of_c[0] = add_atom(g, 6, zero, -1, -1);
  for (int i = 0; i < 4; ++i) {
    double p[3];
    if (i < g->nkids[0]) {
      const int ch = g->kids[i];
      for (int a = 0; a < 3; ++a) p[a] = CC_BOND * tdir[i][a];
      g->idx_of_c[ch] = add_atom(g, 6, p, g->idx_of_c[0], -1);
      for (int a = 0; a < 3; ++a) g->ref[3 * ch + a] = CC_BOND * tdir[(i + 1) % 4][a];
    } else {
      for (int a = 0; a < 3; ++a) p[a] = CH_BOND * tdir[i][a];
      add_atom(g, 1, p, g->idx_of_c[0], -1);
    }
  }
  const int norder = n - 1;
  if (norder > 0) g->start_count[0] = g->count;
  double* cand = (double*)malloc(sizeof(double) * 9 * attempts);
  int* far = (int*)malloc(sizeof(int) * g->total);
  long long draws = 0;
  int t = 0, ok = 0;
  while (t < norder) {
    if (draws >= budget) break;
    const int c = g->order[t];
    g->count = g->start_count[t];
    const int ic = g->idx_of_c[c], ip = g->idx_of_c[g->parent[c]];
    const int nk = g->nkids[c];
    draws += attempts;
    double bc[3], nv[3], mv[3], tmp[3];
    sub3(g->pos + 3 * ic, g->pos + 3 * ip, bc);
    unit3(bc);
    sub3(g->pos + 3 * ip, g->ref + 3 * c, tmp);
    cross3(tmp, bc, nv);
    unit3(nv);
    cross3(nv, bc, mv);
    for (int k = 0; k < attempts; ++k) {
      const double phi = 2.0 * M_PI * uniform01(r);
      for (int s = 0; s < 3; ++s) {
        const double bond = s < nk ? CC_BOND : CH_BOND;
        const double tor = phi + s * (2.0 * M_PI / 3.0);
        const double cs = cos(tor), sn = sin(tor);
        for (int a = 0; a < 3; ++a)
          cand[9 * k + 3 * s + a] = g->pos[3 * ic + a] - bond * ct * bc[a] + bond * st * (cs * mv[a] + sn * nv[a]);
      }
    }
    int nfar = 0;
    const unsigned short* Dic = g->D + (size_t)ic * g->total;
    for (int j = 0; j < g->count; ++j)
      if (Dic[j] + 1 >= 3) far[nfar++] = j;
    /* the draw whose closest approach to a floor is largest (max-min margin);
     * clash-free when that margin is >= 0 */
    int good = -1, back = 0;
    double best = -1e300;
    for (int k = 0; k < attempts; ++k) {
      double margin = 1e300;
      int owner_k = 0;
      for (int s = 0; s < 3; ++s) {
        const double* p = cand + 9 * k + 3 * s;
        for (int f = 0; f < nfar; ++f) {
          const int j = far[f];
          const double lim = (s < nk && g->Z[j] == 6) ? min_cc : min_other;
          const double dx = p[0] - g->pos[3 * j], dy = p[1] - g->pos[3 * j + 1], dz = p[2] - g->pos[3 * j + 2];
          const double d2 = dx * dx + dy * dy + dz * dz;
          const double mg = d2 - lim * lim;
          if (mg < margin) { margin = mg; }
          if (mg < 0.0 && g->owner[j] > owner_k) owner_k = g->owner[j];
        }
      }
      if (margin > best) { best = margin; good = k; }
      if (owner_k > back) back = owner_k;
    }
    if (best < 0.0) good = -1;
    if (good < 0) {   /* back to the latest carbon that placed a clashing atom (root atoms: the first) */
      t = back;
      continue;
    }
    const double* cd = cand + 9 * good;
    for (int s = 0; s < 3; ++s) {
      if (s < nk) {
        const int ch = g->kids[KB(c) + s];
        g->idx_of_c[ch] = add_atom(g, 6, cd + 3 * s, ic, t);
        memcpy(g->ref + 3 * ch, g->pos + 3 * ip, 3 * sizeof(double));
      } else {
        add_atom(g, 1, cd + 3 * s, ic, t);
      }
    }
    ++t;
    if (t < norder) g->start_count[t] = g->count;
  }
  ok = (t >= norder);
  free(cand);
  free(far);
  return ok;
}

/* Returns the number of atoms written (3 n + 2), or -1 when max_trees trees
 * produced no clash-free geometry within `budget` draws each, -2 on bad
 * arguments.  xyz in Angstrom. */
int alkane_generate(unsigned long long seed, int n, double min_cc, double min_other, int attempts,
                    long long budget, int max_trees, int* Z_out, double* xyz_out, int max_atoms) {
  if (n < 1 || attempts < 1 || 3 * n + 2 > max_atoms) return -2;
  rng_t r;
  uint64_t sm = (uint64_t)seed;
  for (int k = 0; k < 4; ++k) r.s[k] = splitmix64(&sm);
  grow_t g;
  memset(&g, 0, sizeof(g));
  g.n = n;
  g.total = 3 * n + 2;
  g.parent = (int*)calloc(n, sizeof(int));
  g.nkids = (int*)calloc(n, sizeof(int));
  g.kids = (int*)calloc(3 * (size_t)n + 4, sizeof(int));   /* 4 + 3 (n - 1) used */
  g.order = (int*)calloc(n, sizeof(int));
  g.idx_of_c = (int*)calloc(n, sizeof(int));
  g.start_count = (int*)calloc(n, sizeof(int));
  g.ref = (double*)calloc(3 * (size_t)n, sizeof(double));
  g.Z = (int*)calloc(g.total, sizeof(int));
  g.pos = (double*)calloc(3 * (size_t)g.total, sizeof(double));
  g.owner = (int*)calloc(g.total, sizeof(int));
  g.D = (unsigned short*)calloc((size_t)g.total * g.total, sizeof(unsigned short));
  int* deg = (int*)calloc(n, sizeof(int));
  int* cand = (int*)calloc(n, sizeof(int));
  int result = -1;
  for (int tree = 0; tree < max_trees && result < 0; ++tree) {
    /* topology */
    memset(g.nkids, 0, n * sizeof(int));
    memset(deg, 0, n * sizeof(int));
    g.parent[0] = -1;
    for (int k = 1; k < n; ++k) {
      int nc = 0;
      for (int c = 0; c < k; ++c) if (deg[c] < 4) cand[nc++] = c;
      const int p = cand[uniform_int(&r, nc)];
      g.parent[k] = p;
      deg[p]++;
      deg[k] = 1;
      g.kids[KB(p) + g.nkids[p]++] = k;
    }
    if (grow(&g, &r, min_cc, min_other, attempts, budget)) {
      for (int i = 0; i < g.count; ++i) {
        Z_out[i] = g.Z[i];
        memcpy(xyz_out + 3 * i, g.pos + 3 * i, 3 * sizeof(double));
      }
      result = g.count;
    }
  }
  free(deg); free(cand);
  free(g.parent); free(g.nkids); free(g.kids); free(g.order); free(g.idx_of_c); free(g.start_count);
  free(g.ref); free(g.Z); free(g.pos); free(g.owner); free(g.D);
  return result;
}
