/*
 * topology_oracle.c -- the reference's geometry reader and wire topology builder,
 * restated in plain C.  TEST INFRASTRUCTURE ONLY: tests/ and the CPU legs of
 * bench.py use it (through oracle/oracle.py) to build the topology arrays of the
 * CPU reference path without the product library; nothing in the product links
 * or loads it.
 *
 * It follows, step by step:
 *   geoinp()      "wersja referencyjna/Configuration.cpp":5-75   (.geo text -> nodes, wires)
 *   configwire()  "wersja referencyjna/Configuration.cpp":112-520 (nodes, wires -> segments,
 *                 basis functions, junctions, PEC-ground virtual wires, 1->0-based shift)
 * keeping the reference's float32 arithmetic (subdivision x0 + j*dx in float) and its
 * array conventions: 0-based storage holding 1-based numbers, second columns at
 * offset nsmax, ipc negative for junction basis functions.  The configwire.txt
 * listing is not produced here.
 *
 * Pinned by tests/test_oracle_golden.py against the arrays of the reference's own
 * config() (tests/golden/topology_*.npz, generated from the reference sources).
 * Compile with -ffp-contract=off (no fused multiply-add), like the reference's
 * scalar float code on x86-64.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* error codes of oracle_topology() */
enum { TOPO_OK = 0, TOPO_PARSE = 1, TOPO_NODES = 2, TOPO_WIRES = 3, TOPO_PATCHES = 4, TOPO_NEGZ = 5,
       TOPO_SEGMENTS = 6, TOPO_BASIS = 7, TOPO_NOMEM = 8 };

/* ------------------------------------------------------------ .geo reader ---- */
/* Cursor over whitespace-separated tokens after the two comment lines. */
typedef struct {
  const char* p;
} tok_cursor;

static int next_int(tok_cursor* c, int* out) {
  char* end;
  long v = strtol(c->p, &end, 10);
  if (end == c->p) return 0;
  c->p = end;
  *out = (int)v;
  return 1;
}

static int next_float(tok_cursor* c, float* out) {
  char* end;
  float v = strtof(c->p, &end);
  if (end == c->p) return 0;
  c->p = end;
  *out = v;
  return 1;
}

/* Configuration.cpp:22-24: the first two lines are comments. */
static const char* skip_two_lines(const char* s) {
  for (int k = 0; k < 2; ++k) {
    const char* nl = strchr(s, '\n');
    if (!nl) return s + strlen(s);
    s = nl + 1;
  }
  return s;
}

/* ------------------------------------------------------------ builder ---- */
/* 1-based work arrays of the topology (the reference's x, y, z, rad, ise, isp, ips,
 * ipc, iwe before the shift of Configuration.cpp:497-514), one slot of margin so that
 * the shift can read index nsmax (resp. 2*nsmax) as the reference does. */
typedef struct {
  int nsmax, nwmax;
  float *x, *y, *z, *rad;
  int *ise, *isp, *ips, *ipc, *iwe;
  int nseg, np, npnt;
} topo_work;

static int seg_new(topo_work* t) {
  if (++t->nseg > t->nsmax) return TOPO_SEGMENTS; /* Configuration.cpp:237-243 */
  return TOPO_OK;
}

static int basis_new(topo_work* t) {
  if (++t->np > t->nsmax - t->nwmax) return TOPO_BASIS; /* Configuration.cpp:248-254 */
  return TOPO_OK;
}

/*
 * Builds the topology of nvw (virtual + real) wires whose node numbers iwnv[m],
 * iwnv[m + nvw] index xnodv/ynodv/znodv, as configwire()'s main loop does
 * (Configuration.cpp:219-488).  Wire m first joins an earlier wire at its start node
 * (the first earlier wire, in order, whose start or end node it shares: the junction
 * segment and junction basis function), then lays its ns segments (float subdivision)
 * and the basis functions between them, then joins an earlier wire at its end node.
 */
static int build_wires(topo_work* t, int nvw, const float* xnodv, const float* ynodv, const float* znodv,
                       const int* iwnv, const float* wradv, const int* nswv) {
  const int S = t->nsmax;
  int i = 0;
  int st;
  for (int m = 1; m <= nvw; ++m) {
    int joined = 0;
    const int ns = nswv[m];
    const int a = iwnv[m], b = iwnv[m + nvw];
    float dx = xnodv[b] - xnodv[a];
    float dy = ynodv[b] - ynodv[a];
    float dz = znodv[b] - znodv[a];
    if (ns > 1) {
      dx = dx / ns;
      dy = dy / ns;
      dz = dz / ns;
    }
    /* junction at the start node (connections 1 and 2, :231-288) */
    for (int n = 1; n < m; ++n) {
      if (a == iwnv[n] || a == iwnv[n + nvw]) {
        const int at_start = (a == iwnv[n]);
        joined = 1;
        if ((st = seg_new(t)) != TOPO_OK) return st;
        if (at_start) {
          /* reversed copy of wire n's first segment */
          t->ise[t->nseg] = t->ise[t->iwe[n] + S];
          t->ise[t->nseg + S] = t->ise[t->iwe[n]];
        } else {
          /* copy of wire n's last segment */
          t->ise[t->nseg] = t->ise[t->iwe[n + S]];
          t->ise[t->nseg + S] = t->ise[t->iwe[n + S] + S];
        }
        t->rad[t->nseg] = wradv[n];
        if ((st = basis_new(t)) != TOPO_OK) return st;
        t->ipc[t->np] = -t->ise[t->nseg + S];
        t->isp[t->nseg] = 0;
        t->isp[t->nseg + S] = t->np;
        t->ips[t->np] = t->nseg;
        break;
      }
    }
    /* the wire's own first node, unless it is the junction's (:290-296) */
    if (!joined) {
      ++i;
      t->x[i] = xnodv[a];
      t->y[i] = ynodv[a];
      t->z[i] = znodv[a];
    }
    /* its segments (:298-327) */
    for (int j = 1; j <= ns; ++j) {
      ++i;
      if (j == ns) {
        t->x[i] = xnodv[b];
        t->y[i] = ynodv[b];
        t->z[i] = znodv[b];
      } else {
        t->x[i] = xnodv[a] + j * dx;
        t->y[i] = ynodv[a] + j * dy;
        t->z[i] = znodv[a] + j * dz;
      }
      if ((st = seg_new(t)) != TOPO_OK) return st;
      t->rad[t->nseg] = wradv[m];
      if (j == 1) t->iwe[m] = joined ? t->nseg - 1 : t->nseg;
      t->ise[t->nseg] = joined ? t->ise[t->nseg - 1 + S] : i - 1;
      t->ise[t->nseg + S] = i;
      t->isp[t->nseg] = 0;
      t->isp[t->nseg + S] = 0;
    }
    /* basis functions between consecutive segments (:329-352); with a start junction
     * the first one is the junction's function, already counted */
    const int mfrst = t->iwe[m];
    int mlast = mfrst + ns - 2;
    if (joined) {
      ++mlast;
      --t->np;
    }
    for (int n = mfrst; n <= mlast; ++n) {
      if ((st = basis_new(t)) != TOPO_OK) return st;
      t->isp[n + S] = t->np;
      t->isp[n + 1] = t->np;
      t->ips[t->np] = n;
      t->ips[t->np + S] = n + 1;
      if (!(joined && n == mfrst)) t->ipc[t->np] = t->ise[n + S];
    }
    t->iwe[m + S] = t->nseg;
    /* junction at the end node (connections 3 and 4, :356-421): one more segment, a
     * copy of the other wire's touching segment, and the basis function across it */
    for (int n = 1; n < m; ++n) {
      if (b == iwnv[n] || b == iwnv[n + nvw]) {
        const int at_start = (b == iwnv[n]);
        if ((st = seg_new(t)) != TOPO_OK) return st;
        --i;
        if (at_start) {
          t->ise[t->nseg] = t->ise[t->iwe[n]];
          t->ise[t->nseg + S] = t->ise[t->iwe[n] + S];
        } else {
          t->ise[t->nseg] = t->ise[t->iwe[n + S] + S];
          t->ise[t->nseg + S] = t->ise[t->iwe[n + S]];
        }
        t->rad[t->nseg] = wradv[n];
        if ((st = basis_new(t)) != TOPO_OK) return st;
        t->ipc[t->np] = -t->ise[t->nseg];
        t->isp[t->iwe[m + S] + S] = t->np;
        t->isp[t->nseg] = t->np;
        t->isp[t->nseg + S] = 0;
        t->ips[t->np] = t->iwe[m + S];
        t->ips[t->np + S] = t->nseg;
        t->ise[t->iwe[m + S] + S] = abs(t->ipc[t->np]);
        t->iwe[m + S] = t->nseg;
        break;
      }
    }
  }
  t->npnt = i;
  return TOPO_OK;
}

/*
 * geo_text: the .geo file's text.  ienv: 1 free space, 2 PEC ground at z = 0.
 * Outputs (caller-owned, zero-initialised by this call): x, y, z, rad, ipc of nsmax
 * entries; ise, isp, ips, iwe of 2*nsmax.  counts[0..3] = npnt, npls, nseg, nw.
 * Limits as the reference driver sets them: nnmax nodes, nwmax wires, ntmax
 * patches (Wire_MoM.cu:43-44).  Returns TOPO_OK or an error code.
 */
int oracle_topology(const char* geo_text, int ienv, int nsmax, int nwmax, int nnmax, int ntmax, float* x,
                    float* y, float* z, float* rad, int* ipc, int* ips, int* ise, int* isp, int* iwe, int* counts) {
  tok_cursor c = {skip_two_lines(geo_text)};
  int nnod = 0, nw = 0, nt = 0;
  int st = TOPO_OK;
  memset(x, 0, sizeof(float) * nsmax);
  memset(y, 0, sizeof(float) * nsmax);
  memset(z, 0, sizeof(float) * nsmax);
  memset(rad, 0, sizeof(float) * nsmax);
  memset(ipc, 0, sizeof(int) * nsmax);
  memset(ise, 0, sizeof(int) * 2 * (size_t)nsmax);
  memset(isp, 0, sizeof(int) * 2 * (size_t)nsmax);
  memset(ips, 0, sizeof(int) * 2 * (size_t)nsmax);
  memset(iwe, 0, sizeof(int) * 2 * (size_t)nsmax);
  memset(counts, 0, 4 * sizeof(int));
  /* geoinp (:26-73): nodes, wires (second node column at offset nw), patches */
  if (!next_int(&c, &nnod) || nnod < 0) return TOPO_PARSE;
  if (nnod > nnmax) return TOPO_NODES;
  float* xnod = calloc((size_t)nnod + 2, sizeof(float));
  float* ynod = calloc((size_t)nnod + 2, sizeof(float));
  float* znod = calloc((size_t)nnod + 2, sizeof(float));
  int* iwn = NULL;
  float* wrad = NULL;
  int* nsw = NULL;
  float *xnodv = NULL, *ynodv = NULL, *znodv = NULL, *wradv = NULL;
  int *iwnv = NULL, *nswv = NULL;
  topo_work t;
  memset(&t, 0, sizeof(t));
  if (!xnod || !ynod || !znod) {
    st = TOPO_NOMEM;
    goto done;
  }
  for (int i = 1; i <= nnod; ++i)
    if (!next_float(&c, &xnod[i]) || !next_float(&c, &ynod[i]) || !next_float(&c, &znod[i])) {
      st = TOPO_PARSE;
      goto done;
    }
  if (!next_int(&c, &nw) || nw < 0) {
    st = TOPO_PARSE;
    goto done;
  }
  if (nw > nwmax) {
    st = TOPO_WIRES;
    goto done;
  }
  iwn = calloc(2 * (size_t)nw + 2, sizeof(int));
  wrad = calloc((size_t)nw + 2, sizeof(float));
  nsw = calloc((size_t)nw + 2, sizeof(int));
  if (!iwn || !wrad || !nsw) {
    st = TOPO_NOMEM;
    goto done;
  }
  for (int i = 1; i <= nw; ++i)
    if (!next_int(&c, &iwn[i]) || !next_int(&c, &iwn[i + nw]) || !next_float(&c, &wrad[i]) ||
        !next_int(&c, &nsw[i])) {
      st = TOPO_PARSE;
      goto done;
    }
  if (!next_int(&c, &nt)) nt = 0;
  if (nt > ntmax) {
    st = TOPO_PATCHES;
    goto done;
  }
  for (int i = 1; i <= nw; ++i)
    if (iwn[i] < 1 || iwn[i] > nnod || iwn[i + nw] < 1 || iwn[i + nw] > nnod || nsw[i] < 1) {
      st = TOPO_PARSE;
      goto done;
    }
  if (nw == 0) goto done; /* :118-124: no wires, nothing built */

  /* PEC ground: no node below z = 0 (:127-144); one virtual wire of one segment,
   * dl long along +x, per (node on the ground, wire touching it) (:146-199) */
  int nadnod = 0, nvnod, nvw;
  if (ienv == 2) {
    for (int i = 1; i <= nnod; ++i)
      if (znod[i] < 0.f) {
        st = TOPO_NEGZ;
        goto done;
      }
    for (int i = 1; i <= nnod; ++i)
      if (fabsf(znod[i]) < 1.e-6) ++nadnod;
  }
  nvnod = nadnod + nnod;
  nvw = nadnod + nw;
  xnodv = calloc((size_t)nvnod + 2, sizeof(float));
  ynodv = calloc((size_t)nvnod + 2, sizeof(float));
  znodv = calloc((size_t)nvnod + 2, sizeof(float));
  wradv = calloc((size_t)nvw + 2, sizeof(float));
  iwnv = calloc(2 * (size_t)nvw + 2, sizeof(int));
  nswv = calloc((size_t)nvw + 2, sizeof(int));
  if (!xnodv || !ynodv || !znodv || !wradv || !iwnv || !nswv) {
    st = TOPO_NOMEM;
    goto done;
  }
  int ivn = 0, ivw = 0;
  if (ienv == 2) {
    for (int i = 1; i <= nnod; ++i) {
      if (!(fabsf(znod[i]) < 1.e-6)) continue;
      for (int j = 1; j <= nw; ++j) {
        if (iwn[j] != i && iwn[j + nw] != i) continue;
        /* the reference counts one virtual node per ground node but adds one per
         * touching wire; keep within the arrays it sized */
        if (ivn + 1 > nadnod || ivw + 1 > nvw) {
          st = TOPO_PARSE;
          goto done;
        }
        ++ivn;
        ++ivw;
        const float ddx = xnod[iwn[j + nw]] - xnod[iwn[j]];
        const float ddy = ynod[iwn[j + nw]] - ynod[iwn[j]];
        const float ddz = znod[iwn[j + nw]] - znod[iwn[j]];
        const float dl = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz) / nsw[j];
        xnodv[ivn] = xnod[i] + dl;
        ynodv[ivn] = ynod[i];
        znodv[ivn] = znod[i];
        iwnv[ivw] = i + nadnod;
        iwnv[ivw + nvw] = ivn;
        wradv[ivw] = wrad[j];
        nswv[ivw] = 1;
      }
    }
  }
  /* real nodes after the virtual ones, real wires after the virtual ones (:202-220) */
  for (int i = 1; i <= nnod; ++i) {
    xnodv[ivn + i] = xnod[i];
    ynodv[ivn + i] = ynod[i];
    znodv[ivn + i] = znod[i];
  }
  for (int i = 1; i <= nw; ++i) {
    iwnv[ivw + i] = iwn[i] + nadnod;
    iwnv[ivw + i + nvw] = iwn[i + nw] + nadnod;
    wradv[ivw + i] = wrad[i];
    nswv[ivw + i] = nsw[i];
  }

  t.nsmax = nsmax;
  t.nwmax = nwmax;
  t.x = calloc((size_t)nsmax + 2, sizeof(float));
  t.y = calloc((size_t)nsmax + 2, sizeof(float));
  t.z = calloc((size_t)nsmax + 2, sizeof(float));
  t.rad = calloc((size_t)nsmax + 2, sizeof(float));
  t.ipc = calloc((size_t)nsmax + 2, sizeof(int));
  t.ise = calloc(2 * (size_t)nsmax + 2, sizeof(int));
  t.isp = calloc(2 * (size_t)nsmax + 2, sizeof(int));
  t.ips = calloc(2 * (size_t)nsmax + 2, sizeof(int));
  t.iwe = calloc(2 * (size_t)nsmax + 2, sizeof(int));
  if (!t.x || !t.y || !t.z || !t.rad || !t.ipc || !t.ise || !t.isp || !t.ips || !t.iwe) {
    st = TOPO_NOMEM;
    goto done;
  }
  /* more wires than virtual-wire slots never reach build_wires: nvw >= nw */
  if ((st = build_wires(&t, nvw, xnodv, ynodv, znodv, iwnv, wradv, nswv)) != TOPO_OK) goto done;

  /* the shift to 0-based storage (:497-514), in place and in the reference's order:
   * entry k-1 takes entry k for k = 1..nsmax in both halves, so the first half's
   * last slot ends up holding the second half's first entry */
  for (int k = 1; k <= nsmax; ++k) {
    t.x[k - 1] = t.x[k];
    t.y[k - 1] = t.y[k];
    t.z[k - 1] = t.z[k];
    t.ise[k - 1] = t.ise[k];
    t.ise[k - 1 + nsmax] = t.ise[k + nsmax];
    t.isp[k - 1] = t.isp[k];
    t.isp[k - 1 + nsmax] = t.isp[k + nsmax];
    t.iwe[k - 1] = t.iwe[k];
    t.iwe[k - 1 + nsmax] = t.iwe[k + nsmax];
    t.rad[k - 1] = t.rad[k];
    t.ips[k - 1] = t.ips[k];
    t.ips[k - 1 + nsmax] = t.ips[k + nsmax];
    t.ipc[k - 1] = t.ipc[k];
  }
  memcpy(x, t.x, sizeof(float) * nsmax);
  memcpy(y, t.y, sizeof(float) * nsmax);
  memcpy(z, t.z, sizeof(float) * nsmax);
  memcpy(rad, t.rad, sizeof(float) * nsmax);
  memcpy(ipc, t.ipc, sizeof(int) * nsmax);
  memcpy(ise, t.ise, sizeof(int) * 2 * (size_t)nsmax);
  memcpy(isp, t.isp, sizeof(int) * 2 * (size_t)nsmax);
  memcpy(ips, t.ips, sizeof(int) * 2 * (size_t)nsmax);
  memcpy(iwe, t.iwe, sizeof(int) * 2 * (size_t)nsmax);
  counts[0] = t.npnt;
  counts[1] = t.np;
  counts[2] = t.nseg;
  counts[3] = nw;

done:
  free(xnod);
  free(ynod);
  free(znod);
  free(iwn);
  free(wrad);
  free(nsw);
  free(xnodv);
  free(ynodv);
  free(znodv);
  free(wradv);
  free(iwnv);
  free(nswv);
  free(t.x);
  free(t.y);
  free(t.z);
  free(t.rad);
  free(t.ipc);
  free(t.ise);
  free(t.isp);
  free(t.ips);
  free(t.iwe);
  return st;
}
