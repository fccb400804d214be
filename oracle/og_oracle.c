/*
 * FP64 CPU oracle for the GIMIC current-density hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference's algorithm, used by tests/, by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py as the checker.  Nothing in the shipped package
 * (gimic_gb300/) links, imports or calls it.
 *
 * Every routine names the reference routine it restates (paths are relative to
 * the GIMIC source tree).  Arithmetic is IEEE double throughout and loop orders
 * follow the reference so that results can be compared point by point.
 *
 * Parity pins: the oracle is checked against the reference's committed outputs
 * (test/c4h4/read-grid jvec.vtu, test/c4h4/integration stdout,
 * test/open-shell/integration stdout, test/open-shell/3d *.vti) by
 * tests/test_oracle_golden.py.
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OG_MAX_L 5
#define OG_MAXLINE 4096

/* ---------------------------------------------------------------------------
 * Cartesian component tables: src/libgimic/gtodefs.f90:86-123.
 * Standard order and TURBOMOLE order (symlib/pdfgtr.f ordering).
 * ------------------------------------------------------------------------- */
static const int GT_STD[6][21][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 2, 0}, {0, 1, 1}, {0, 0, 2}},
    {{3, 0, 0}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {1, 1, 1}, {1, 0, 2}, {0, 3, 0}, {0, 2, 1}, {0, 1, 2}, {0, 0, 3}},
    {{4, 0, 0}, {3, 1, 0}, {3, 0, 1}, {2, 2, 0}, {2, 1, 1}, {2, 0, 2}, {1, 3, 0}, {1, 2, 1},
     {1, 1, 2}, {1, 0, 3}, {0, 4, 0}, {0, 3, 1}, {0, 2, 2}, {0, 1, 3}, {0, 0, 4}},
    {{5, 0, 0}, {4, 1, 0}, {4, 0, 1}, {3, 2, 0}, {3, 1, 1}, {3, 0, 2}, {2, 3, 0}, {2, 2, 1}, {2, 1, 2}, {2, 0, 3},
     {1, 4, 0}, {1, 3, 1}, {1, 2, 2}, {1, 1, 3}, {1, 0, 4}, {0, 5, 0}, {0, 4, 1}, {0, 3, 2}, {0, 2, 3}, {0, 1, 4}, {0, 0, 5}},
};
static const int GT_TM[6][21][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
    {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {0, 2, 1}, {1, 0, 2}, {0, 1, 2}, {1, 1, 1}},
    {{4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {1, 3, 0}, {0, 3, 1}, {1, 0, 3},
     {0, 1, 3}, {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2}},
    {{5, 0, 0}, {0, 5, 0}, {0, 0, 5}, {4, 1, 0}, {4, 0, 1}, {1, 4, 0}, {0, 4, 1}, {1, 0, 4}, {0, 1, 4}, {3, 2, 0},
     {3, 0, 2}, {2, 3, 0}, {0, 3, 2}, {2, 0, 3}, {0, 2, 3}, {3, 1, 1}, {1, 3, 1}, {1, 1, 3}, {2, 2, 1}, {2, 1, 2}, {1, 2, 2}},
};

typedef struct {
    int l, npf, ncomp;
    double *xp, *cc, *ncc;
    double thrs; /* screening radius (basis%thrs) */
    int pos;     /* first function of this contraction within its atom (basis%pos) */
} og_ctr;

typedef struct {
    double coord[3];
    double charge;
    char symbol[3];
    int nshells;
    int nctrps[OG_MAX_L + 1];
    int nctr;
    og_ctr *ctr;
    int ncgto; /* functions on this atom */
} og_atom;

typedef struct {
    int natoms, ncgto, ngto, turbomole, uhf;
    og_atom *atoms;
    int *fatom;      /* atom of each function */
    /* spherical basis (Advanced.spherical): nfun = nsph functions of 2l+1
     * components per shell; c2s[s * ncgto + c] projects Cartesian component
     * c onto spherical function s (cao2sao_t%po, cao2sao.f90:64-101) */
    int spherical, nfun;
    double *c2s;
    int *fatom_s;
    double *da, *db; /* [4][n*n] column-major: D, dD/dBx, dD/dBy, dD/dBz */
    int giao, dia, para;
    char err[512];
} og_ctx;

typedef struct {
    double origin[3];
    double basv[9]; /* basv(:,d) at basv[3*d] */
    int npts[3];
    const double *pts[3];
    const double *wgt[3];
    double radius;
} og_grid;

/* ---------------------------------------------------------------------------
 * Fortran list-directed reading (enough of it for INTGRL and XDENS files):
 * every READ starts on a new record, takes values across records as needed,
 * skips blank records, and discards what is left of its last record.
 * ------------------------------------------------------------------------- */
typedef struct {
    FILE *f;
    char line[OG_MAXLINE];
    char *p;   /* cursor within line; NULL when the line is exhausted */
    int eof;
} og_rd;

static int rd_nextline(og_rd *r) {
    if (!fgets(r->line, sizeof r->line, r->f)) {
        r->eof = 1;
        r->p = NULL;
        return 0;
    }
    r->p = r->line;
    return 1;
}

/* start a new READ statement: the next record */
static int rd_begin(og_rd *r) { return rd_nextline(r); }

static int rd_token(og_rd *r, char *tok, size_t n) {
    for (;;) {
        if (r->p == NULL) {
            if (!rd_nextline(r)) return 0;
        }
        while (*r->p && (isspace((unsigned char)*r->p) || *r->p == ',')) r->p++;
        if (*r->p == '\0') {
            r->p = NULL;
            continue;
        }
        size_t k = 0;
        while (*r->p && !isspace((unsigned char)*r->p) && *r->p != ',') {
            if (k + 1 < n) tok[k++] = *r->p;
            r->p++;
        }
        tok[k] = '\0';
        return 1;
    }
}

static int rd_double(og_rd *r, double *v) {
    char tok[128];
    if (!rd_token(r, tok, sizeof tok)) return 0;
    for (char *c = tok; *c; c++)
        if (*c == 'd' || *c == 'D') *c = 'E';
    char *end;
    *v = strtod(tok, &end);
    return end != tok;
}

static int rd_int(og_rd *r, int *v) {
    double d;
    if (!rd_double(r, &d)) return 0;
    *v = (int)d;
    return 1;
}

/* ---------------------------------------------------------------------------
 * src/libgimic/basis.f90:164-191 (norm_ctr)
 * ------------------------------------------------------------------------- */
static void norm_ctr(og_ctr *c) {
    double j = 1.0 * (c->l + 1);
    double n = 0.0;
    for (int l = 0; l < c->npf; l++) {
        double c1 = c->cc[l], e1 = c->xp[l];
        for (int m = 0; m <= l; m++) {
            double e2 = c->xp[m], c2 = c->cc[m];
            double t = 2.0 * sqrt(e1 * e2) / (e1 + e2);
            t = c1 * c2 * pow(t, j + 0.5);
            n = n + t;
            if (l != m) n = n + t;
        }
    }
    n = 1.0 / sqrt(n);
    for (int l = 0; l < c->npf; l++) {
        double c1 = c->cc[l], e1 = c->xp[l];
        c->ncc[l] = c1 * n * pow(4.0 * e1, 0.5 * j + 0.25) * pow(0.5 / 3.141592653589793, 0.75);
    }
}

/* src/libgimic/basis.f90:90-112 (setup_screening) */
static double ipow(double x, int l) {
    double r = 1.0;
    for (int i = 0; i < l; i++) r *= x;
    return r;
}
static void setup_screening(og_atom *a, double thrs) {
    for (int i = 0; i < a->nctr; i++) {
        og_ctr *c = &a->ctr[i];
        double min_xp = 1e15, x = 1e15, dist = 0.0;
        for (int j = 0; j < c->npf; j++)
            if (c->xp[j] < min_xp) min_xp = c->xp[j];
        while (x > thrs) {
            dist = dist + 0.25;
            x = ipow(dist, c->l) * exp(-min_xp * dist * dist);
        }
        c->thrs = dist;
    }
}

/* ---------------------------------------------------------------------------
 * src/libgimic/intgrl.f90:20-264 (read_intgrl, read_atom, read_segs,
 * read_contraction2, get_basdim) and basis.f90:29-86, 216-249.
 * ------------------------------------------------------------------------- */
static int read_intgrl(og_ctx *x, const char *fname, double screen_thrs) {
    og_rd r = {0};
    r.f = fopen(fname, "r");
    if (!r.f) {
        snprintf(x->err, sizeof x->err, "read_intgrl(): open failed: %s", fname);
        return -1;
    }
    if (!rd_nextline(&r) || strncmp(r.line, "INTGRL", 6) != 0) {
        snprintf(x->err, sizeof x->err, "not an INTGRL file: %s", fname);
        fclose(r.f);
        return -1;
    }
    rd_nextline(&r);
    x->turbomole = strncmp(r.line, "TURBOMOLE", 9) == 0;
    rd_nextline(&r); /* title line */
    rd_begin(&r);
    int natoms;
    if (!rd_int(&r, &natoms) || natoms <= 0) {
        snprintf(x->err, sizeof x->err, "bad atom count");
        fclose(r.f);
        return -1;
    }
    rd_nextline(&r); /* line 5 */
    x->natoms = natoms;
    x->atoms = calloc((size_t)natoms, sizeof(og_atom));
    for (int a = 0; a < natoms; a++) {
        og_atom *at = &x->atoms[a];
        double charge;
        int dummy, nsh;
        rd_begin(&r);
        if (!rd_double(&r, &charge) || !rd_int(&r, &dummy) || !rd_int(&r, &nsh)) goto bad;
        if (nsh - 1 > OG_MAX_L || nsh < 1) {
            snprintf(x->err, sizeof x->err, "Largest allowed l-quantum number in basis exceeded: %d", nsh - 1);
            fclose(r.f);
            return -1;
        }
        int nctrps[OG_MAX_L + 1];
        for (int i = 0; i < nsh; i++)
            if (!rd_int(&r, &nctrps[i])) goto bad;
        at->charge = charge;
        at->nshells = nsh;
        /* read_atom: symbol in columns 1-2, id in 3-4, coordinates after */
        if (!rd_nextline(&r)) goto bad;
        at->symbol[0] = r.line[0];
        at->symbol[1] = r.line[1] ? r.line[1] : ' ';
        at->symbol[2] = '\0';
        if (strlen(r.line) < 5) goto bad;
        r.p = r.line + 4;
        for (int d = 0; d < 3; d++)
            if (!rd_double(&r, &at->coord[d])) goto bad;
        /* read_segs: general contractions split into segments (ncf copies) */
        int cap = 64, nctr = 0;
        og_ctr *ctr = calloc((size_t)cap, sizeof(og_ctr));
        for (int i = 0; i < nsh; i++) {
            int nseg = 0;
            for (int j = 0; j < nctrps[i]; j++) {
                int npf, ncf;
                rd_begin(&r);
                if (!rd_int(&r, &npf) || !rd_int(&r, &ncf) || npf < 1 || ncf < 1) goto bad;
                if (nctr + ncf > cap) {
                    cap = 2 * (nctr + ncf);
                    ctr = realloc(ctr, (size_t)cap * sizeof(og_ctr));
                }
                for (int k = 0; k < ncf; k++) {
                    og_ctr *c = &ctr[nctr + k];
                    memset(c, 0, sizeof *c);
                    c->l = i;
                    c->npf = npf;
                    c->ncomp = (i + 1) * (i + 2) / 2;
                    c->xp = calloc((size_t)npf, sizeof(double));
                    c->cc = calloc((size_t)npf, sizeof(double));
                    c->ncc = calloc((size_t)npf, sizeof(double));
                }
                for (int p = 0; p < npf; p++) {
                    double xp;
                    rd_begin(&r);
                    if (!rd_double(&r, &xp)) goto bad;
                    for (int k = 0; k < ncf; k++) {
                        double cc;
                        if (!rd_double(&r, &cc)) goto bad;
                        ctr[nctr + k].xp[p] = xp;
                        ctr[nctr + k].cc[p] = cc;
                    }
                }
                nctr += ncf;
                nseg += ncf;
            }
            at->nctrps[i] = nseg;
        }
        at->nctr = nctr;
        at->ctr = ctr;
    }
    fclose(r.f);
    /* calc_basdim (basis.f90:216-249) and normalisation */
    x->ncgto = 0;
    x->ngto = 0;
    for (int a = 0; a < natoms; a++) {
        og_atom *at = &x->atoms[a];
        at->ncgto = 0;
        for (int k = 0; k < at->nctr; k++) {
            at->ctr[k].pos = at->ncgto;
            at->ncgto += at->ctr[k].ncomp;
            x->ngto += at->ctr[k].npf * at->ctr[k].ncomp;
            norm_ctr(&at->ctr[k]);
        }
        x->ncgto += at->ncgto;
        if (screen_thrs <= 0.0) {
            for (int k = 0; k < at->nctr; k++) at->ctr[k].thrs = 1e10;
        } else {
            setup_screening(at, screen_thrs);
        }
    }
    x->fatom = malloc((size_t)x->ncgto * sizeof(int));
    int q = 0;
    for (int a = 0; a < natoms; a++)
        for (int k = 0; k < x->atoms[a].ncgto; k++) x->fatom[q++] = a;
    return 0;
bad:
    snprintf(x->err, sizeof x->err, "malformed INTGRL file: %s", fname);
    fclose(r.f);
    return -1;
}

/* ---------------------------------------------------------------------------
 * src/libgimic/reorder.f90:54-96 (turbo_reorder): sv(q) = atom-major index of
 * the q-th function when functions are listed by l first.
 * ------------------------------------------------------------------------- */
static void turbo_sv(const og_ctx *x, int *sv) {
    int n = x->ncgto;
    int *lvec = malloc((size_t)n * sizeof(int));
    int q = 0;
    for (int a = 0; a < x->natoms; a++) {
        const og_atom *at = &x->atoms[a];
        for (int k = 0; k < at->nctr; k++)
            for (int c = 0; c < at->ctr[k].ncomp; c++) lvec[q++] = at->ctr[k].l;
    }
    int l = 0;
    q = 0;
    while (q < n) {
        for (int i = 0; i < n; i++)
            if (lvec[i] == l) sv[q++] = i;
        l++;
    }
    free(lvec);
}

/* src/libgimic/dens.f90:56-135 (read_dens, read_array), :210-234 (reorder_dens) */
static int read_dens(og_ctx *x, const char *fname) {
    int n = x->nfun;
    size_t nn = (size_t)n * n;
    og_rd r = {0};
    r.f = fopen(fname, "r");
    if (!r.f) {
        snprintf(x->err, sizeof x->err, "Density file not found: %s", fname);
        return -1;
    }
    x->da = calloc(4 * nn, sizeof(double));
    if (x->uhf) x->db = calloc(4 * nn, sizeof(double));
    for (int s = 0; s < (x->uhf ? 2 : 1); s++) {
        double *dens = s == 0 ? x->da : x->db;
        for (size_t i = 0; i < 4 * nn; i++) {
            rd_begin(&r);
            if (!rd_double(&r, &dens[i])) {
                snprintf(x->err, sizeof x->err, "XDENS file too short: %s", fname);
                fclose(r.f);
                return -1;
            }
        }
    }
    fclose(r.f);
    if (x->uhf) {
        for (size_t i = nn; i < 4 * nn; i++) {
            x->da[i] = x->da[i] / 2.0;
            x->db[i] = x->db[i] / 2.0;
        }
    }
    if (x->turbomole) {
        int *sv = malloc((size_t)n * sizeof(int));
        turbo_sv(x, sv);
        double *tmp = malloc(nn * sizeof(double));
        for (int s = 0; s < (x->uhf ? 2 : 1); s++) {
            double *dens = s == 0 ? x->da : x->db;
            for (int b = 0; b < 4; b++) {
                double *m = dens + b * nn;
                /* new(sv(i), sv(j)) = old(i, j) */
                for (int j = 0; j < n; j++)
                    for (int i = 0; i < n; i++) tmp[sv[i] + (size_t)sv[j] * n] = m[i + (size_t)j * n];
                memcpy(m, tmp, nn * sizeof(double));
            }
        }
        free(tmp);
        free(sv);
    }
    return 0;
}

/* ---------------------------------------------------------------------------
 * Basis functions: src/libgimic/caos.f90:17-110 (cgto, dcgto, cao, cao2) and
 * src/libgimic/bfeval.f90:81-122 (bfeval), :295-338 (dfdr), :168-189 (mkdbop),
 * :271-293 (dfdb), :191-246 (d2fdrdb).
 * ------------------------------------------------------------------------- */
static double prod_pow(const double r[3], const int f[3]) {
    return pow(r[0], (double)f[0]) * pow(r[1], (double)f[1]) * pow(r[2], (double)f[2]);
}

static void basis_point(const og_ctx *x, const double r[3], double *bf, double *dr) {
    int n = x->ncgto;
    const int(*gt)[21][3] = x->turbomole ? GT_TM : GT_STD;
    memset(bf, 0, (size_t)n * sizeof(double));
    if (dr) memset(dr, 0, 3 * (size_t)n * sizeof(double));
    int idx2 = 0;
    for (int a = 0; a < x->natoms; a++) {
        const og_atom *at = &x->atoms[a];
        double rr[3] = {r[0] - at->coord[0], r[1] - at->coord[1], r[2] - at->coord[2]};
        double dist = sqrt(rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2]);
        double rr2 = rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2];
        for (int k = 0; k < at->nctr; k++) {
            const og_ctr *c = &at->ctr[k];
            if (!(dist <= c->thrs)) continue; /* filter_screened */
            int idx = idx2 + c->pos;
            /* cgto */
            double q = 0.0;
            for (int p = 0; p < c->npf; p++) q = q + c->ncc[p] * exp(-c->xp[p] * rr2);
            for (int i = 0; i < c->ncomp; i++) bf[idx + i] = prod_pow(rr, gt[c->l][i]) * q;
            if (!dr) continue;
            /* dcgto for the three axes (cao2) */
            double bfval = 0.0, dbfval = 0.0;
            for (int p = 0; p < c->npf; p++) {
                double qq = c->ncc[p] * exp(-c->xp[p] * rr2);
                bfval = bfval + qq;
                dbfval = dbfval + c->xp[p] * qq;
            }
            for (int ax = 0; ax < 3; ax++) {
                for (int i = 0; i < c->ncomp; i++) {
                    const int *f = gt[c->l][i];
                    int df[3] = {f[0], f[1], f[2]};
                    df[ax] = df[ax] - 1;
                    if (df[ax] < 0) df[ax] = 0;
                    double down = (double)f[ax] * prod_pow(rr, df) * bfval;
                    double up = 2.0 * rr[ax] * prod_pow(rr, f) * dbfval;
                    dr[idx + i + (size_t)ax * n] = down - up;
                }
            }
        }
        idx2 += at->ncgto;
    }
}

/* ---------------------------------------------------------------------------
 * src/libgimic/jtensor.F90:105-123 (jtensor) and :148-237 (contract), the
 * matmul (non-BLAS) branch: denbf = matmul(bf, D), pdbf = matmul(bf, P_b),
 * dendb = matmul(db(:,b), D).  ct is 3x3 column-major, ct(m,b) at m+3b.
 * ------------------------------------------------------------------------- */
typedef struct {
    double *bf, *dr, *db, *d2, *denbf, *dendb, *pdbf;
    double *bfc, *drc; /* Cartesian values before the spherical projection */
} og_work;

static og_work work_new(int n, int ncart) {
    og_work w;
    w.bfc = calloc((size_t)ncart, sizeof(double));
    w.drc = calloc(3 * (size_t)ncart, sizeof(double));
    w.bf = calloc((size_t)n, sizeof(double));
    w.dr = calloc(3 * (size_t)n, sizeof(double));
    w.db = calloc(3 * (size_t)n, sizeof(double));
    w.d2 = calloc(9 * (size_t)n, sizeof(double));
    w.denbf = calloc((size_t)n, sizeof(double));
    w.dendb = calloc((size_t)n, sizeof(double));
    w.pdbf = calloc((size_t)n, sizeof(double));
    return w;
}
static void work_free(og_work *w) {
    free(w->bfc);
    free(w->drc);
    free(w->bf);
    free(w->dr);
    free(w->db);
    free(w->d2);
    free(w->denbf);
    free(w->dendb);
    free(w->pdbf);
}

static void vec_mat(int n, const double *v, const double *m, double *out) {
    for (int j = 0; j < n; j++) {
        const double *col = m + (size_t)j * n;
        double s = 0.0;
        for (int i = 0; i < n; i++) s += v[i] * col[i];
        out[j] = s;
    }
}
static double dot(int n, const double *a, const double *b) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

static void jtensor_spin(const og_ctx *x, og_work *w, const double r[3], int spin, double ct[9], double *rho_out) {
    int n = x->nfun;
    size_t nn = (size_t)n * n;
    const double *dens = spin == 1 ? x->db : x->da;
    double rho[3] = {0.5 * r[0], 0.5 * r[1], 0.5 * r[2]};
    const int *fatom = x->spherical ? x->fatom_s : x->fatom;
    if (x->spherical) {
        /* bfeval.f90:116-117 and dfdr, :330-333: sbf = matmul(po, bf) */
        int nc = x->ncgto;
        basis_point(x, r, w->bfc, w->drc);
        for (int s = 0; s < n; s++) {
            const double *row = x->c2s + (size_t)s * nc;
            double v = 0.0, g[3] = {0.0, 0.0, 0.0};
            for (int c = 0; c < nc; c++) {
                if (row[c] == 0.0) continue;
                v += row[c] * w->bfc[c];
                for (int ax = 0; ax < 3; ax++) g[ax] += row[c] * w->drc[c + (size_t)ax * nc];
            }
            w->bf[s] = v;
            for (int ax = 0; ax < 3; ax++) w->dr[s + (size_t)ax * n] = g[ax];
        }
    } else {
        basis_point(x, r, w->bf, w->dr);
    }
    if (x->giao) {
        /* mkdbop + dfdb + d2fdrdb */
        for (int mu = 0; mu < n; mu++) {
            const double *R = x->atoms[fatom[mu]].coord;
            double dbop[3] = {r[1] * R[2] - r[2] * R[1], r[2] * R[0] - r[0] * R[2], r[0] * R[1] - r[1] * R[0]};
            double bfv = w->bf[mu];
            double dx = w->dr[mu], dy = w->dr[mu + n], dz = w->dr[mu + 2 * (size_t)n];
            for (int b = 0; b < 3; b++) w->db[mu + (size_t)b * n] = dbop[b] * bfv;
            double *d2 = w->d2;
            d2[mu + 0 * (size_t)n] = dx * dbop[0];
            d2[mu + 1 * (size_t)n] = dy * dbop[0] + R[2] * bfv;
            d2[mu + 2 * (size_t)n] = dz * dbop[0] - R[1] * bfv;
            d2[mu + 3 * (size_t)n] = dx * dbop[1] - R[2] * bfv;
            d2[mu + 4 * (size_t)n] = dy * dbop[1];
            d2[mu + 5 * (size_t)n] = dz * dbop[1] + R[0] * bfv;
            d2[mu + 6 * (size_t)n] = dx * dbop[2] + R[1] * bfv;
            d2[mu + 7 * (size_t)n] = dy * dbop[2] - R[0] * bfv;
            d2[mu + 8 * (size_t)n] = dz * dbop[2];
        }
    }
    vec_mat(n, w->bf, dens, w->denbf);
    double diapam = dot(n, w->denbf, w->bf);
    if (rho_out) *rho_out = diapam;
    double dpd[3];
    int k = 0;
    for (int b = 0; b < 3; b++) {
        vec_mat(n, w->bf, dens + (size_t)(b + 1) * nn, w->pdbf);
        if (x->giao) vec_mat(n, w->db + (size_t)b * n, dens, w->dendb);
        dpd[b] = diapam * rho[b];
        for (int m = 0; m < 3; m++) {
            double prsp1 = 0.0, prsp2 = 0.0;
            if (x->giao) {
                prsp1 = -dot(n, w->dendb, w->dr + (size_t)m * n);
                prsp2 = dot(n, w->denbf, w->d2 + (size_t)k * n);
            }
            double ppd = dot(n, w->pdbf, w->dr + (size_t)m * n);
            ct[m + 3 * b] = 0.5 * ppd;
            if (x->giao) ct[m + 3 * b] = ct[m + 3 * b] + 0.5 * (prsp1 + prsp2);
            k++;
        }
    }
    if (!x->para)
        for (int i = 0; i < 9; i++) ct[i] = 0.0;
    if (!x->dia) dpd[0] = dpd[1] = dpd[2] = 0.0;
    ct[0 + 3 * 1] += dpd[2];
    ct[0 + 3 * 2] -= dpd[1];
    ct[1 + 3 * 0] -= dpd[2];
    ct[1 + 3 * 2] += dpd[0];
    ct[2 + 3 * 0] += dpd[1];
    ct[2 + 3 * 1] -= dpd[0];
}

/* spin case codes: 0 total, 1 alpha, 2 beta, 3 spindens */
static int spin_code(const char *s) {
    if (!s || !strcmp(s, "total")) return 0;
    if (!strcmp(s, "alpha")) return 1;
    if (!strcmp(s, "beta")) return 2;
    if (!strcmp(s, "spindens")) return 3;
    return -1;
}

/* src/libgimic/jtensor.F90:66-103 (ctensor) */
static int ctensor(const og_ctx *x, og_work *w, const double r[3], int sc, double j[9], double *rho) {
    double j1[9], j2[9], r1 = 0, r2 = 0;
    switch (sc) {
        case 1:
            jtensor_spin(x, w, r, 0, j, rho);
            return 0;
        case 2:
            if (!x->uhf) return -2;
            jtensor_spin(x, w, r, 1, j, rho);
            return 0;
        case 0:
            if (x->uhf) {
                jtensor_spin(x, w, r, 0, j1, &r1);
                jtensor_spin(x, w, r, 1, j2, &r2);
                for (int i = 0; i < 9; i++) j[i] = j1[i] + j2[i];
                if (rho) *rho = r1 + r2;
            } else {
                jtensor_spin(x, w, r, 0, j, rho);
            }
            return 0;
        case 3:
            if (!x->uhf) return -3;
            jtensor_spin(x, w, r, 0, j1, &r1);
            jtensor_spin(x, w, r, 1, j2, &r2);
            for (int i = 0; i < 9; i++) j[i] = j1[i] - j2[i];
            if (rho) *rho = r1 - r2;
            return 0;
    }
    return -1;
}

/* ---------------------------------------------------------------------------
 * Quadrature: src/libgimic/gaussint.f90:21-59 (gaussl), :61-112 (lobattomy),
 * :144-222 (legendrep1/2), :267-319 (setup_gauss_data).
 * ------------------------------------------------------------------------- */
static void legendrep1(double x, int n, double *y, double *dy) {
    *y = 1.0;
    *dy = 0.0;
    if (n == 0) return;
    *y = x;
    *dy = 1.0;
    if (n == 1) return;
    double yp = 1.0, dyp = 0.0;
    for (int i = 2; i <= n; i++) {
        double c1 = (double)i, c2 = c1 * 2.0 - 1.0, c4 = c1 - 1.0;
        double ym = *y;
        *y = (c2 * x * *y - c4 * yp) / c1;
        yp = ym;
        double dym = *dy;
        *dy = (c2 * x * *dy - c4 * dyp + c2 * yp) / c1;
        dyp = dym;
    }
}
static void legendrep2(double x, int n, double *y, double *dy, double *d2y) {
    *y = 1.0;
    *dy = 0.0;
    *d2y = 0.0;
    if (n == 0) return;
    *y = x;
    *dy = 1.0;
    *d2y = 0.0;
    if (n == 1) return;
    double yp = 1.0, dyp = 0.0, d2yp = 0.0;
    for (int i = 2; i <= n; i++) {
        double c1 = (double)i, c2 = c1 * 2.0 - 1.0, c4 = c1 - 1.0;
        double ym = *y;
        *y = (c2 * x * *y - c4 * yp) / c1;
        yp = ym;
        double dym = *dy;
        *dy = (c2 * x * *dy - c4 * dyp + c2 * yp) / c1;
        dyp = dym;
        double d2ym = *d2y;
        *d2y = (c2 * x * *d2y - c4 * d2yp + c2 * 2.0 * dyp) / c1;
        d2yp = d2ym;
    }
}
#define OG_PII 3.141592653589793
#define OG_EPS 3.0e-12
#define OG_NEWTON_MAX 10

static int gaussl(double a, double b, int n, double *pts, double *wgt) {
    int m = (n % 2 == 0) ? n / 2 : (n + 1) / 2;
    double xm = (b + a) * 0.5, xl = (b - a) * 0.5;
    for (int i = 1; i <= m; i++) {
        double z = cos(OG_PII * ((double)i - 0.25) / ((double)n + 0.5)), z1, lp = 0, dlp = 0;
        int iter;
        for (iter = 1; iter <= OG_NEWTON_MAX; iter++) {
            legendrep1(z, n, &lp, &dlp);
            z1 = z;
            z = z1 - lp / dlp;
            if (fabs(z - z1) <= OG_EPS) break;
        }
        if (iter >= OG_NEWTON_MAX) return -1;
        pts[i - 1] = xm - xl * z;
        pts[n - i] = xm + xl * z;
        wgt[i - 1] = 2.0 * xl / ((1.0 - z * z) * dlp * dlp);
        wgt[n - i] = wgt[i - 1];
    }
    return 0;
}

static int lobattomy(double a, double b, int n, double *pts, double *wgt) {
    double xm = (b + a) * 0.5, xl = (b - a) * 0.5;
    pts[0] = xm - xl;
    pts[n - 1] = xm + xl;
    wgt[0] = 2.0 * xl / (double)(n * n - n);
    wgt[n - 1] = wgt[0];
    for (int i = 2; i <= n - 1; i++) {
        double z = cos(OG_PII * ((double)i - 0.25) / ((double)n + 0.5)), z1, lp = 0, dlp = 0, d2lp = 0;
        int iter;
        for (iter = 1; iter <= OG_NEWTON_MAX; iter++) {
            legendrep2(z, n - 1, &lp, &dlp, &d2lp);
            z1 = z;
            z = z1 - dlp / d2lp;
            double damp = 0.5;
            while (fabs(z) > 1.0) {
                z = z1 - dlp / d2lp * damp;
                damp = damp * damp;
            }
            if (fabs(z - z1) <= OG_EPS) break;
        }
        if (iter >= OG_NEWTON_MAX) return -1;
        pts[i - 1] = xm - xl * z;
        wgt[i - 1] = 2.0 * xl / ((double)(n * n - n) * lp * lp);
    }
    return 0;
}

/* setup_gauss_data(a, b, ngp, gdata, quadr) with size(gdata%pts) = npts.
 * quadr: 0 gauss, 1 lobatto.  Note the points start at 0, as in the reference. */
int og_gauss_data(double a, double b, int ngp, int npts, int quadr, double *pts, double *wgt) {
    if (npts == 1) {
        pts[0] = 0.0;
        wgt[0] = 1.0;
        return 0;
    }
    if (ngp <= 0 || npts % ngp != 0) return -1;
    int nblock = npts / ngp;
    double step = (b - a) / (double)nblock;
    double xl = step * 0.5;
    double *tp = malloc((size_t)ngp * sizeof(double)), *tw = malloc((size_t)ngp * sizeof(double));
    int rc = quadr == 1 ? lobattomy(-1.0, 1.0, ngp, tp, tw) : gaussl(-1.0, 1.0, ngp, tp, tw);
    if (rc == 0) {
        for (int j = 0; j < ngp; j++) tp[j] = tp[j] + 1.0;
        int foo = 0;
        for (int i = 1; i <= nblock; i++) {
            for (int j = 0; j < ngp; j++) {
                pts[foo + j] = tp[j] * xl + (double)(i - 1) * step;
                wgt[foo + j] = tw[j] * xl;
            }
            foo += ngp;
        }
    }
    free(tp);
    free(tw);
    return rc;
}

/* ---------------------------------------------------------------------------
 * Cartesian -> spherical projection, src/libgimic/cao2sao.f90: mkc2sop
 * (:173-201), clmtuv (:153-170), renorm (:205-235), assembled per shell by
 * new_c2sop (:64-101).  Rows run over m = -l..l (the sphmap reordering is
 * commented out in the reference, :187).  As in the reference each (t, u, v)
 * term is ASSIGNED to its Cartesian component; for l <= 3 no two terms share
 * a component, so the rows are the exact real solid harmonics, rescaled by
 * renorm to integer coefficients (d: xy, yz, 2zz - xx - yy, xz, xx - yy).
 * The normalisation nslm drops out in renorm and is not restated.
 * ------------------------------------------------------------------------- */
static long og_fact(int n) {
    long m = 1;
    for (int i = 2; i <= n; i++) m *= i;
    return m;
}
static long og_binom(int a, int b) { return og_fact(a) / (og_fact(b) * og_fact(a - b)); }

static int gt_index(int l, int i, int j, int k) {
    for (int c = 0; c < (l + 1) * (l + 2) / 2; c++)
        if (GT_STD[l][c][0] == i && GT_STD[l][c][1] == j && GT_STD[l][c][2] == k) return c;
    return -1;
}

static void renorm_row(double *row, int nc) {
    double amin = 1e10;
    for (int j = 0; j < nc; j++) {
        double ava = fabs(row[j]);
        if (ava > 0.0 && ava < amin) amin = ava;
    }
    for (int j = 0; j < nc; j++) row[j] /= amin;
    double sim = 1.0;
    for (int j = 0; j < nc; j++) {
        double ava = fabs(row[j]);
        if (!(ava > 0.0)) continue;
        double avb = fmod(ava, 1.0);
        if (avb > 1e-10) {
            ava = 1.0 / avb;
            while (fmod(ava, 1.0) > 1e-10) {
                avb = fmod(ava, 1.0);
                if (avb > 1e-10) ava = ava / avb;
            }
            if (ava > sim) sim = ava;
        }
    }
    for (int j = 0; j < nc; j++) row[j] *= sim;
}

/* xop[(2l+1) x ncart] row-major */
static void mkc2sop(int l, double *xop) {
    int nc = (l + 1) * (l + 2) / 2;
    memset(xop, 0, (size_t)(2 * l + 1) * nc * sizeof(double));
    for (int m = -l; m <= l; m++) {
        double *row = xop + (size_t)(m + l) * nc;
        int am = m < 0 ? -m : m;
        double vm = m < 0 ? 0.5 : 0.0;
        for (int t = 0; t <= (l - am) / 2; t++)
            for (int u = 0; u <= t; u++)
                for (int v = 0; v <= (int)(am * 0.5 - vm); v++) {
                    double vr = v + vm;
                    int i = 2 * t + am - (int)(2.0 * (u + vr));
                    int j = (int)(2.0 * (u + vr));
                    int k = l - 2 * t - am;
                    double q = 1.0 / pow(4.0, t);
                    if (fmod((double)t + vr - vm, 2.0) > 0.0) q = -q;
                    q *= (double)(og_binom(l, t) * og_binom(l - t, am + t) * og_binom(t, u) * og_binom(am, (int)(2.0 * vr)));
                    int n = gt_index(l, i, j, k);
                    if (n >= 0) row[n] = q;
                }
        renorm_row(row, nc);
    }
}

static int setup_spherical(og_ctx *x) {
    if (x->turbomole) {
        snprintf(x->err, sizeof x->err, "spherical basis with TURBOMOLE component order is not supported");
        return -1;
    }
    int ns = 0;
    for (int a = 0; a < x->natoms; a++)
        for (int k = 0; k < x->atoms[a].nctr; k++) ns += 2 * x->atoms[a].ctr[k].l + 1;
    x->nfun = ns;
    x->c2s = calloc((size_t)ns * x->ncgto, sizeof(double));
    x->fatom_s = malloc((size_t)ns * sizeof(int));
    double xop[11 * 21];
    int srow = 0, ccol = 0;
    for (int a = 0; a < x->natoms; a++) {
        const og_atom *at = &x->atoms[a];
        for (int k = 0; k < at->nctr; k++) {
            int l = at->ctr[k].l, nc = (l + 1) * (l + 2) / 2;
            mkc2sop(l, xop);
            for (int s = 0; s < 2 * l + 1; s++) {
                for (int c = 0; c < nc; c++) x->c2s[(size_t)(srow + s) * x->ncgto + ccol + at->ctr[k].pos + c] = xop[s * nc + c];
                x->fatom_s[srow + s] = a;
            }
            srow += 2 * l + 1;
        }
        ccol += at->ncgto;
    }
    return 0;
}

/* ---------------------------------------------------------------------------
 * Public API (ctypes)
 * ------------------------------------------------------------------------- */
static void og_free_atoms(og_ctx *x) {
    if (!x->atoms) return;
    for (int a = 0; a < x->natoms; a++) {
        og_atom *at = &x->atoms[a];
        for (int k = 0; k < at->nctr; k++) {
            free(at->ctr[k].xp);
            free(at->ctr[k].cc);
            free(at->ctr[k].ncc);
        }
        free(at->ctr);
    }
    free(x->atoms);
    x->atoms = NULL;
}

void og_free(og_ctx *x) {
    if (!x) return;
    og_free_atoms(x);
    free(x->fatom);
    free(x->fatom_s);
    free(x->c2s);
    free(x->da);
    free(x->db);
    free(x);
}

/* Load MOL (+ XDENS unless xdens is NULL).  screen_thrs <= 0 disables
 * screening (basis%thrs = 1e10), as in basis.f90:69-73. */
og_ctx *og_load_sph(const char *mol, const char *xdens, int uhf, double screen_thrs, int spherical, char *err,
                    int errlen) {
    og_ctx *x = calloc(1, sizeof(og_ctx));
    x->uhf = uhf != 0;
    x->giao = x->dia = x->para = 1;
    int rc = read_intgrl(x, mol, screen_thrs);
    x->nfun = x->ncgto;
    x->spherical = spherical != 0;
    if (rc == 0 && x->spherical) rc = setup_spherical(x);
    if (rc == 0 && xdens) rc = read_dens(x, xdens);
    if (rc != 0) {
        if (err && errlen > 0) snprintf(err, (size_t)errlen, "%s", x->err);
        og_free(x);
        return NULL;
    }
    return x;
}

og_ctx *og_load(const char *mol, const char *xdens, int uhf, double screen_thrs, char *err, int errlen) {
    return og_load_sph(mol, xdens, uhf, screen_thrs, 0, err, errlen);
}

int og_ncgto(const og_ctx *x) { return x->ncgto; }
/* functions the densities are given in: spherical or Cartesian */
int og_nfun(const og_ctx *x) { return x->nfun; }
/* the projection, nfun x ncgto row-major (spherical contexts only) */
int og_c2s(const og_ctx *x, double *out) {
    if (!x->spherical) return -1;
    memcpy(out, x->c2s, (size_t)x->nfun * x->ncgto * sizeof(double));
    return 0;
}
int og_ngto(const og_ctx *x) { return x->ngto; }
int og_natoms(const og_ctx *x) { return x->natoms; }
int og_is_turbomole(const og_ctx *x) { return x->turbomole; }
void og_atom_info(const og_ctx *x, int a, double *coord, double *charge) {
    for (int d = 0; d < 3; d++) coord[d] = x->atoms[a].coord[d];
    *charge = x->atoms[a].charge;
}
void og_set_flags(og_ctx *x, int giao, int dia, int para) {
    x->giao = giao;
    x->dia = dia;
    x->para = para;
}
/* spin 0 alpha (or closed shell), 1 beta; b 0 = D, 1..3 = dD/dB */
int og_get_dens(const og_ctx *x, int spin, int b, double *out) {
    const double *d = spin == 1 ? x->db : x->da;
    if (!d) return -1;
    size_t nn = (size_t)x->nfun * x->nfun;
    memcpy(out, d + (size_t)b * nn, nn * sizeof(double));
    return 0;
}
/* Shell table: for each contraction (atom-major): atom, l, npf, pos, thrs. */
int og_nctr_total(const og_ctx *x) {
    int s = 0;
    for (int a = 0; a < x->natoms; a++) s += x->atoms[a].nctr;
    return s;
}
void og_shell_table(const og_ctx *x, int *atom, int *l, int *npf, int *pos, double *thrs, double *xp, double *ncc,
                    int maxprim) {
    int s = 0;
    for (int a = 0; a < x->natoms; a++)
        for (int k = 0; k < x->atoms[a].nctr; k++) {
            const og_ctr *c = &x->atoms[a].ctr[k];
            atom[s] = a;
            l[s] = c->l;
            npf[s] = c->npf;
            pos[s] = c->pos;
            thrs[s] = c->thrs;
            for (int p = 0; p < maxprim; p++) {
                xp[(size_t)s * maxprim + p] = p < c->npf ? c->xp[p] : 0.0;
                ncc[(size_t)s * maxprim + p] = p < c->npf ? c->ncc[p] : 0.0;
            }
            s++;
        }
}

/* basis values and gradients at one point: bf[n], dr[n*3] (column per axis) */
void og_basis_eval(const og_ctx *x, const double r[3], double *bf, double *dr) { basis_point(x, r, bf, dr); }

/* ctensor at npts points r[3*i]; jt[9*i] column-major; rho[i] optional.
 * Returns 0, or a negative spin error (beta/spindens on a closed shell). */
int og_jtensor_batch(const og_ctx *x, const char *spin, long npts, const double *r, double *jt, double *rho,
                     int nthreads) {
    int sc = spin_code(spin);
    if (sc < 0) return -1;
    if (!x->uhf && (sc == 2 || sc == 3)) return -2;
    int err = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
    {
        og_work w = work_new(x->nfun, x->ncgto);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (long i = 0; i < npts; i++) {
            double rv = 0;
            err |= ctensor(x, &w, r + 3 * i, sc, jt + 9 * i, &rv) != 0;
            if (rho) rho[i] = rv;
        }
        work_free(&w);
    }
    (void)nthreads;
    return err ? -3 : 0;
}

/* src/libgimic/acid.f90:11-43 (get_acid); DP33 = 0.3333333 as in globals.f90:62 */
double og_acid(const double *t) {
    double xxmyy = (t[0] - t[4]) * (t[0] - t[4]);
    double yymzz = (t[4] - t[8]) * (t[4] - t[8]);
    double zzmxx = (t[8] - t[0]) * (t[8] - t[0]);
    double xypyx = (t[3] + t[1]) * (t[3] + t[1]);
    double xzpzx = (t[6] + t[2]) * (t[6] + t[2]);
    double yzpzy = (t[7] + t[5]) * (t[7] + t[5]);
    return 0.3333333 * (xxmyy + yymzz + zzmxx) + 0.5 * (xypyx + xzpzx + yzpzy);
}

/* src/libgimic/globals.f90 au2si */
double og_au2si(double au) {
    double aulength = 0.52917726e-10, auspeedoflight = 137.03599, speedoflight = 299792458.0;
    double aucharge = 1.60217733e-19, hbar = 1.05457267e-34;
    double autime = aulength * auspeedoflight / speedoflight;
    double autesla = hbar / aucharge / aulength / aulength;
    double audjdb = aucharge / autime / autesla;
    return au * audjdb * 1.0e9;
}

static void gridpoint(const og_grid *g, int i, int j, int k, double r[3]) {
    for (int d = 0; d < 3; d++)
        r[d] = g->origin[d] + g->pts[0][i] * g->basv[d] + g->pts[1][j] * g->basv[3 + d] + g->pts[2][k] * g->basv[6 + d];
}

/* Plane/volume integrals, src/fgimic/integral.f90:50-186 (integrate_current),
 * :190-324 (integrate_modulus), :414-511 (integrate_acid).
 * what: 0 current, 1 modulus, 2 acid.  out: {total, positive, negative} in au
 * (acid: {sqrt(sum), sum, 0}).  Rows j are summed in order; the reference's
 * OpenMP split of j changes only the order of the row partial sums. */
int og_integrate(const og_ctx *x, const char *spin, const og_grid *g, const double bb[3], int what, double out[3],
                 int nthreads) {
    int sc = spin_code(spin);
    if (sc < 0) return -1;
    if (!x->uhf && (sc == 2 || sc == 3)) return -2;
    int p1 = g->npts[0], p2 = g->npts[1], p3 = g->npts[2];
    const double *normal = g->basv + 6;
    double center[3], v1[3], v2[3];
    gridpoint(g, p1 - 1, 0, 0, v1);
    gridpoint(g, 0, p2 - 1, 0, v2);
    for (int d = 0; d < 3; d++) center[d] = (v1[d] + v2[d]) * 0.5;
    double bound = g->radius;
    double xsum3 = 0, psum3 = 0, nsum3 = 0;
    double *rowx = malloc((size_t)p2 * sizeof(double));
    double *rowp = malloc((size_t)p2 * sizeof(double));
    double *rown = malloc((size_t)p2 * sizeof(double));
    (void)nthreads;
    for (int k = 0; k < p3; k++) {
#ifdef _OPENMP
        if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
        {
            og_work w = work_new(x->nfun, x->ncgto);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (int j = 0; j < p2; j++) {
                double xsum = 0, psum = 0, nsum = 0, sgn = 1.0;
                for (int i = 0; i < p1; i++) {
                    double rr[3], tt[9], jvec[3];
                    gridpoint(g, i, j, k, rr);
                    double dx = rr[0] - center[0], dy = rr[1] - center[1], dz = rr[2] - center[2];
                    double r = sqrt(dx * dx + dy * dy + dz * dz);
                    ctensor(x, &w, rr, sc, tt, NULL);
                    for (int m = 0; m < 3; m++) jvec[m] = tt[m] * bb[0] + tt[m + 3] * bb[1] + tt[m + 6] * bb[2];
                    if (what == 0) {
                        double wt, jp;
                        if (r > bound) {
                            wt = 0.0;
                            jp = 0.0;
                        } else {
                            wt = g->wgt[0][i];
                            jp = (normal[0] * jvec[0] + normal[1] * jvec[1] + normal[2] * jvec[2]) * wt;
                        }
                        (void)wt;
                        xsum = xsum + jp;
                        if (jp > 0.0)
                            psum = psum + jp;
                        else
                            nsum = nsum + jp;
                    } else if (what == 1) {
                        double wt;
                        if (r > bound) {
                            wt = 0.0;
                        } else {
                            wt = g->wgt[0][i];
                            double jp = normal[0] * jvec[0] + normal[1] * jvec[1] + normal[2] * jvec[2];
                            if (fabs(jp) < 1e-12)
                                sgn = 0.0;
                            else if (jp > 0)
                                sgn = 1.0;
                            else
                                sgn = -1.0;
                        }
                        double jp = sgn * sqrt(jvec[0] * jvec[0] + jvec[1] * jvec[1] + jvec[2] * jvec[2]);
                        xsum = xsum + jp * wt;
                        if (jp > 0.0)
                            psum = psum + jp * wt;
                        else
                            nsum = nsum + jp * wt;
                    } else {
                        double val = og_acid(tt);
                        double wt = r > bound ? 0.0 : g->wgt[0][i];
                        xsum = xsum + val * wt;
                    }
                }
                double wj = g->wgt[1][j];
                rowx[j] = xsum * wj;
                rowp[j] = psum * wj;
                rown[j] = nsum * wj;
            }
            work_free(&w);
        }
        double xsum2 = 0, psum2 = 0, nsum2 = 0;
        for (int j = 0; j < p2; j++) {
            xsum2 += rowx[j];
            psum2 += rowp[j];
            nsum2 += rown[j];
        }
        double wk = g->wgt[2][k];
        xsum3 = xsum3 + wk * xsum2;
        psum3 = psum3 + wk * psum2;
        nsum3 = nsum3 + wk * nsum2;
    }
    free(rowx);
    free(rowp);
    free(rown);
    if (what == 2) {
        out[0] = sqrt(xsum3);
        out[1] = xsum3;
        out[2] = 0.0;
    } else {
        out[0] = xsum3;
        out[1] = psum3;
        out[2] = nsum3;
    }
    return 0;
}

/* Build an og_grid from caller arrays (ctypes-friendly). */
int og_integrate_flat(const og_ctx *x, const char *spin, const double *origin, const double *basv, const int *npts,
                      const double *p1, const double *w1, const double *p2, const double *w2, const double *p3,
                      const double *w3, double radius, const double *bb, int what, double *out, int nthreads) {
    og_grid g;
    memcpy(g.origin, origin, sizeof g.origin);
    memcpy(g.basv, basv, sizeof g.basv);
    memcpy(g.npts, npts, sizeof g.npts);
    g.pts[0] = p1;
    g.pts[1] = p2;
    g.pts[2] = p3;
    g.wgt[0] = w1;
    g.wgt[1] = w2;
    g.wgt[2] = w3;
    g.radius = radius;
    return og_integrate(x, spin, &g, bb, what, out, nthreads);
}
