/*
 * md_oracle.c -- CPU oracle (test infrastructure only; see md_oracle.h).
 *
 * A plain-C restatement of the reference's short-range MD path.  Each block
 * names the reference function it follows (paths relative to the ls1-mardyn
 * tree).  Arithmetic is written in the operation order of the reference's
 * scalar (no-intrinsics) kernel path, so with -ffp-contract=off every single
 * pair interaction rounds exactly as the reference's does; totals differ from
 * the reference only by summation order.
 */
#include "md_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXC 16
#define MAXS 16

typedef struct {
    int nlj, nch, ndi, nqu, ns;
    double lj[MAXS][7], ch[MAXS][5], di[MAXS][7], qu[MAXS][7];
    double m, I[3], invI[3];
    int rot_dof;
    int ljoff; /* first global LJ-centre index of this component */
} ocomp;

struct orc_sys {
    md_config cfg;
    int ncomp;
    ocomp cdef[MAXC];
    int nlj;                /* LJ centres over all components */
    double *eps24, *sig2, *shift6; /* nlj x nlj, VectorizedCellProcessor.cpp:54-80 */
    double epsRFInvrc3;
    /* grid (LinkedCells.cpp:38-105) */
    int nin[3], cpd[3];
    double cl[3], clr[3], bmin[3], bmax[3], hmin[3], hmax[3];
    double* border[3];
    /* molecules: [0, n) inner, [n, ntot) halo copies */
    int64_t n, ntot, cap;
    uint64_t* id;
    int32_t* mcomp;
    int64_t* orig;
    double *r, *v, *q, *L, *F, *M, *Vi;
    /* site caches (CellDataSoA) */
    int64_t* soff;
    int64_t nsites, scap;
    double *spos, *se, *sF, *sV, *sM;
    /* cells */
    int64_t ncells;
    int64_t *cstart, *clist, *mcell;
    /* global velocity-scaling thermostat (target <= 0: NVE) and the explosion
       heuristic's counters (Domain.cpp:74-76) */
    double thermo_T;
    int thermo_heur, th_counter, th_warning, th_error;
};

static int g_threads = 1;

int orc_set_threads(int32_t n) {
    g_threads = n > 0 ? n : 1;
    return 0;
}

/* ---------------------------------------------------------------- quaternion
 * Quaternion::rotate / rotateinv / differentiate (src/molecules/Quaternion.cpp:43-103). */
static void q_rotate(const double* q, const double* d, double* out) {
    if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) { out[0] = out[1] = out[2] = 0.0; return; }
    double ww = q[0] * q[0], xx = q[1] * q[1], yy = q[2] * q[2], zz = q[3] * q[3];
    double wx = q[0] * q[1], wy = q[0] * q[2], wz = q[0] * q[3];
    double xy = q[1] * q[2], xz = q[1] * q[3], yz = q[2] * q[3];
    out[0] = (ww + xx - yy - zz) * d[0] + 2. * (xy - wz) * d[1] + 2. * (wy + xz) * d[2];
    out[1] = 2. * (wz + xy) * d[0] + (ww - xx + yy - zz) * d[1] + 2. * (yz - wx) * d[2];
    out[2] = 2. * (xz - wy) * d[0] + 2. * (wx + yz) * d[1] + (ww - xx - yy + zz) * d[2];
}

static void q_rotateinv(const double* q, const double* d, double* out) {
    if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) { out[0] = out[1] = out[2] = 0.0; return; }
    double ww = q[0] * q[0], xx = q[1] * q[1], yy = q[2] * q[2], zz = q[3] * q[3];
    double wx = q[0] * q[1], wy = q[0] * q[2], wz = q[0] * q[3];
    double xy = q[1] * q[2], xz = q[1] * q[3], yz = q[2] * q[3];
    out[0] = (ww + xx - yy - zz) * d[0] + 2. * (xy + wz) * d[1] + 2. * (xz - wy) * d[2];
    out[1] = 2. * (xy - wz) * d[0] + (ww - xx + yy - zz) * d[1] + 2. * (yz + wx) * d[2];
    out[2] = 2. * (xz + wy) * d[0] + 2. * (yz - wx) * d[1] + (ww - xx - yy + zz) * d[2];
}

static void q_differentiate(const double* q, const double* w, double* dq) {
    dq[0] = .5 * (-q[1] * w[0] - q[2] * w[1] - q[3] * w[2]);
    dq[1] = .5 * (q[0] * w[0] - q[3] * w[1] + q[2] * w[2]);
    dq[2] = .5 * (q[3] * w[0] + q[0] * w[1] - q[1] * w[2]);
    dq[3] = .5 * (-q[2] * w[0] + q[1] * w[1] + q[0] * w[2]);
}

static double q_mag2(const double* q) { return q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]; }

static void q_scale(double* q, double s) { q[0] *= s; q[1] *= s; q[2] *= s; q[3] *= s; }

/* Quaternion::normalize = scaleinv(sqrt(magnitude2())) = scale(1./sqrt(..)) */
static void q_normalize(double* q) { q_scale(q, 1. / sqrt(q_mag2(q))); }

/* ---------------------------------------------------------------- setup */
orc_sys* orc_create(const md_config* cfg, const md_component* comps, int32_t ncomp, const double* mixing) {
    if (!cfg || !comps || ncomp < 1 || ncomp > MAXC) return NULL;
    orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
    s->cfg = *cfg;
    s->ncomp = ncomp;
    int nlj = 0;
    for (int c = 0; c < ncomp; ++c) {
        ocomp* o = &s->cdef[c];
        const md_component* in = &comps[c];
        if (in->n_lj > MAXS || in->n_charge > MAXS || in->n_dipole > MAXS || in->n_quadrupole > MAXS) {
            free(s);
            return NULL;
        }
        o->nlj = in->n_lj; o->nch = in->n_charge; o->ndi = in->n_dipole; o->nqu = in->n_quadrupole;
        o->ns = o->nlj + o->nch + o->ndi + o->nqu;
        for (int i = 0; i < o->nlj; ++i) memcpy(o->lj[i], in->lj + 7 * i, 7 * sizeof(double));
        for (int i = 0; i < o->nch; ++i) memcpy(o->ch[i], in->charge + 5 * i, 5 * sizeof(double));
        for (int i = 0; i < o->ndi; ++i) memcpy(o->di[i], in->dipole + 7 * i, 7 * sizeof(double));
        for (int i = 0; i < o->nqu; ++i) memcpy(o->qu[i], in->quadrupole + 7 * i, 7 * sizeof(double));
        /* Component::updateMassInertia (src/molecules/Component.cpp:137-178): LJ centres, then charges */
        o->m = 0.0;
        o->I[0] = o->I[1] = o->I[2] = 0.0;
        o->rot_dof = 0;
        for (int k = 0; k < o->nlj + o->nch; ++k) {
            const double* st = k < o->nlj ? o->lj[k] : o->ch[k - o->nlj];
            double m = st[3], x = st[0], y = st[1], z = st[2];
            o->m += m;
            o->I[0] += m * (y * y + z * z);
            o->I[1] += m * (x * x + z * z);
            o->I[2] += m * (x * x + y * y);
            o->rot_dof = 3;
            for (int d = 0; d < 3; ++d)
                if (o->I[d] == 0.) --o->rot_dof;
        }
        /* header inertia overrides (ASCIIReader: setI11/22/33 when > 0) */
        for (int d = 0; d < 3; ++d)
            if (in->inertia[d] > 0.) o->I[d] = in->inertia[d];
        /* FullMolecule::updateMassInertia (src/molecules/FullMolecule.h:88-101) */
        for (int d = 0; d < 3; ++d) o->invI[d] = o->I[d] != 0. ? 1. / o->I[d] : 0.;
        o->ljoff = nlj;
        nlj += o->nlj;
    }
    s->nlj = nlj;
    s->eps24 = (double*)calloc((size_t)(nlj * nlj + 1), sizeof(double));
    s->sig2 = (double*)calloc((size_t)(nlj * nlj + 1), sizeof(double));
    s->shift6 = (double*)calloc((size_t)(nlj * nlj + 1), sizeof(double));
    /* Comp2Param::initialize (src/molecules/Comp2Param.cpp:11-105) */
    int mix = 0;
    for (int ci = 0; ci < ncomp; ++ci) {
        const ocomp* A = &s->cdef[ci];
        for (int i = 0; i < A->nlj; ++i)
            for (int j = 0; j < A->nlj; ++j) {
                double epsi = A->lj[i][4], sigi = A->lj[i][5], epsj = A->lj[j][4], sigj = A->lj[j][5];
                double e24 = 24. * sqrt(epsi * epsj);
                double s2 = .5 * (sigi + sigj);
                s2 *= s2;
                int gi = A->ljoff + i, gj = A->ljoff + j;
                s->eps24[gi * nlj + gj] = e24;
                s->sig2[gi * nlj + gj] = s2;
                s->shift6[gi * nlj + gj] = A->lj[i][6];
            }
        for (int cj = ci + 1; cj < ncomp; ++cj) {
            const ocomp* B = &s->cdef[cj];
            double xi = mixing ? mixing[2 * mix] : 1.0, eta = mixing ? mixing[2 * mix + 1] : 1.0;
            ++mix;
            for (int i = 0; i < A->nlj; ++i)
                for (int j = 0; j < B->nlj; ++j) {
                    double epsi = A->lj[i][4], sigi = A->lj[i][5], epsj = B->lj[j][4], sigj = B->lj[j][5];
                    double e24 = 24. * (xi * sqrt(epsi * epsj));
                    double s2 = 0.5 * (eta * (sigi + sigj));
                    s2 *= s2;
                    double sp2 = s2 / (cfg->rc_lj * cfg->rc_lj);
                    double sp6 = sp2 * sp2 * sp2;
                    double sh = e24 * (sp6 - sp6 * sp6);
                    int gi = A->ljoff + i, gj = B->ljoff + j;
                    s->eps24[gi * nlj + gj] = e24; s->sig2[gi * nlj + gj] = s2; s->shift6[gi * nlj + gj] = sh;
                    s->eps24[gj * nlj + gi] = e24; s->sig2[gj * nlj + gi] = s2; s->shift6[gj * nlj + gi] = sh;
                }
        }
    }
    /* VectorizedCellProcessor ctor (VectorizedCellProcessor.cpp:22) */
    double rc = cfg->rc;
    s->epsRFInvrc3 = 2. * (cfg->eps_rf - 1.) / ((rc * rc * rc) * (2. * cfg->eps_rf + 1.));
    /* LinkedCells::LinkedCells (LinkedCells.cpp:38-75) */
    s->ncells = 1;
    for (int d = 0; d < 3; ++d) {
        s->bmin[d] = cfg->box_min[d];
        s->bmax[d] = cfg->box_max[d];
        int n = (int)floor((s->bmax[d] - s->bmin[d]) / rc);
        if (n == 0) n = 1;
        s->nin[d] = n;
        double diff = s->bmax[d] - s->bmin[d];
        s->cl[d] = diff / n;
        s->clr[d] = n / diff;
        s->hmin[d] = s->bmin[d] - s->cl[d];
        s->hmax[d] = s->bmax[d] + s->cl[d];
        s->cpd[d] = n + 2;
        s->ncells *= s->cpd[d];
        /* CellBorderAndFlagManager::getBorder (CellBorderAndFlagManager.h:134-152) */
        s->border[d] = (double*)malloc(sizeof(double) * (size_t)(s->cpd[d] + 1));
        for (int i = 0; i <= s->cpd[d]; ++i) {
            double b;
            if (i == 0) b = s->hmin[d];
            else if (i == 1) b = s->bmin[d];
            else if (i == s->cpd[d] - 1) b = s->bmax[d];
            else if (i == s->cpd[d]) b = s->hmax[d];
            else b = i * s->cl[d] + s->hmin[d];
            s->border[d][i] = b;
        }
    }
    s->cstart = (int64_t*)calloc((size_t)s->ncells + 1, sizeof(int64_t));
    return s;
}

void orc_destroy(orc_sys* s) {
    if (!s) return;
    free(s->eps24); free(s->sig2); free(s->shift6);
    for (int d = 0; d < 3; ++d) free(s->border[d]);
    free(s->id); free(s->mcomp); free(s->orig);
    free(s->r); free(s->v); free(s->q); free(s->L); free(s->F); free(s->M); free(s->Vi);
    free(s->soff); free(s->spos); free(s->se); free(s->sF); free(s->sV); free(s->sM);
    free(s->cstart); free(s->clist); free(s->mcell);
    free(s);
}

static void reserve(orc_sys* s, int64_t cap) {
    if (cap <= s->cap) return;
    s->id = (uint64_t*)realloc(s->id, sizeof(uint64_t) * cap);
    s->mcomp = (int32_t*)realloc(s->mcomp, sizeof(int32_t) * cap);
    s->orig = (int64_t*)realloc(s->orig, sizeof(int64_t) * cap);
    s->r = (double*)realloc(s->r, sizeof(double) * 3 * cap);
    s->v = (double*)realloc(s->v, sizeof(double) * 3 * cap);
    s->q = (double*)realloc(s->q, sizeof(double) * 4 * cap);
    s->L = (double*)realloc(s->L, sizeof(double) * 3 * cap);
    s->F = (double*)realloc(s->F, sizeof(double) * 3 * cap);
    s->M = (double*)realloc(s->M, sizeof(double) * 3 * cap);
    s->Vi = (double*)realloc(s->Vi, sizeof(double) * 3 * cap);
    s->soff = (int64_t*)realloc(s->soff, sizeof(int64_t) * (cap + 1));
    s->mcell = (int64_t*)realloc(s->mcell, sizeof(int64_t) * cap);
    s->clist = (int64_t*)realloc(s->clist, sizeof(int64_t) * cap);
    s->cap = cap;
}

int orc_set_molecules(orc_sys* s, int64_t n, const uint64_t* id, const int32_t* comp, const double* r,
                      const double* v, const double* q, const double* L) {
    reserve(s, n + 16);
    s->n = s->ntot = n;
    for (int64_t k = 0; k < n; ++k) {
        if (comp[k] < 0 || comp[k] >= s->ncomp) return MD_ERR_ARG;
        s->id[k] = id ? id[k] : (uint64_t)(k + 1);
        s->mcomp[k] = comp[k];
        s->orig[k] = k;
    }
    memcpy(s->r, r, sizeof(double) * 3 * n);
    memcpy(s->v, v, sizeof(double) * 3 * n);
    memcpy(s->q, q, sizeof(double) * 4 * n);
    memcpy(s->L, L, sizeof(double) * 3 * n);
    memset(s->F, 0, sizeof(double) * 3 * n);
    memset(s->M, 0, sizeof(double) * 3 * n);
    memset(s->Vi, 0, sizeof(double) * 3 * n);
    return MD_OK;
}

int64_t orc_num_molecules(const orc_sys* s) { return s->n; }

int orc_set_forces(orc_sys* s, int64_t n, const double* F, const double* M, const double* Vi) {
    if (n != s->n) return MD_ERR_ARG;
    if (F) memcpy(s->F, F, sizeof(double) * 3 * n);
    if (M) memcpy(s->M, M, sizeof(double) * 3 * n);
    if (Vi) memcpy(s->Vi, Vi, sizeof(double) * 3 * n);
    return MD_OK;
}

int orc_get_molecules(const orc_sys* s, int64_t n, uint64_t* id, int32_t* comp, double* r, double* v, double* q,
                      double* L, double* F, double* M, double* Vi) {
    if (n != s->n) return MD_ERR_ARG;
    if (id) memcpy(id, s->id, sizeof(uint64_t) * n);
    if (comp) memcpy(comp, s->mcomp, sizeof(int32_t) * n);
    if (r) memcpy(r, s->r, sizeof(double) * 3 * n);
    if (v) memcpy(v, s->v, sizeof(double) * 3 * n);
    if (q) memcpy(q, s->q, sizeof(double) * 4 * n);
    if (L) memcpy(L, s->L, sizeof(double) * 3 * n);
    if (F) memcpy(F, s->F, sizeof(double) * 3 * n);
    if (M) memcpy(M, s->M, sizeof(double) * 3 * n);
    if (Vi) memcpy(Vi, s->Vi, sizeof(double) * 3 * n);
    return MD_OK;
}

/* ---------------------------------------------------------------- binning
 * LinkedCells::getCellIndexOfPoint (src/particleContainer/LinkedCells.cpp:870-923)
 * with ParticleCellBase::testPointInCell [min, max) (ParticleCellBase.h:66-71). */
static int64_t cell_of_point(const orc_sys* s, const double* point) {
    int ci[3];
    double p[3] = {point[0], point[1], point[2]};
    for (int d = 0; d < 3; ++d) {
        if (p[d] <= s->hmin[d]) p[d] += s->cl[d] * 0.5;
        else if (p[d] >= s->hmax[d]) p[d] -= s->cl[d] * 0.5;
        int c = (int)floor((p[d] - s->bmin[d]) * s->clr[d]) + 1;
        if (c < 0) c = 0;
        if (c > s->cpd[d] - 1) c = s->cpd[d] - 1;
        ci[d] = c;
    }
    int inside = 1;
    for (int d = 0; d < 3; ++d)
        inside &= (s->border[d][ci[d]] <= p[d]) && (p[d] < s->border[d][ci[d] + 1]);
    if (!inside) {
        for (int d = 0; d < 3; ++d) {
            if (p[d] < s->border[d][ci[d]]) ci[d]--;
            else if (p[d] >= s->border[d][ci[d] + 1]) ci[d]++;
        }
    }
    return ((int64_t)ci[2] * s->cpd[1] + ci[1]) * s->cpd[0] + ci[0];
}

static int in_region(const double* r, const double* lo, const double* hi) {
    return r[0] >= lo[0] && r[0] < hi[0] && r[1] >= lo[1] && r[1] < hi[1] && r[2] >= lo[2] && r[2] < hi[2];
}

static int64_t add_copy(orc_sys* s, int64_t k) {
    if (s->ntot + 1 > s->cap) reserve(s, s->cap * 2 + 64);
    int64_t h = s->ntot++;
    s->id[h] = s->id[k]; s->mcomp[h] = s->mcomp[k]; s->orig[h] = s->orig[k];
    memcpy(s->r + 3 * h, s->r + 3 * k, 3 * sizeof(double));
    memcpy(s->v + 3 * h, s->v + 3 * k, 3 * sizeof(double));
    memcpy(s->q + 4 * h, s->q + 4 * k, 4 * sizeof(double));
    memcpy(s->L + 3 * h, s->L + 3 * k, 3 * sizeof(double));
    return h;
}

int orc_rebin_and_halo(orc_sys* s, md_bin_stats* st) {
    const double rc = s->cfg.rc;
    int64_t wrapped = 0;
    s->ntot = s->n;
    /* DomainDecompBase::handleDomainLeavingParticles (DomainDecompBase.cpp:199-249) */
    for (int d = 0; d < 3; ++d) {
        if (!s->cfg.periodic[d]) continue;
        const double L = s->bmax[d] - s->bmin[d];
        for (int dir = 0; dir < 2; ++dir) {
            double lo[3], hi[3];
            for (int e = 0; e < 3; ++e) { lo[e] = s->bmin[e] - rc; hi[e] = s->bmax[e] + rc; }
            if (dir == 0) hi[d] = s->bmin[d]; else lo[d] = s->bmax[d];
            double shift = dir == 0 ? L : -L;
            for (int64_t k = 0; k < s->n; ++k) {
                double* r = s->r + 3 * k;
                if (!in_region(r, lo, hi)) continue;
                r[d] = r[d] + shift;
                if (shift < 0) {
                    if (r[d] <= s->bmin[d]) r[d] = s->bmin[d];
                } else {
                    if (r[d] >= s->bmax[d]) r[d] = nextafter(s->bmax[d], -INFINITY);
                }
                ++wrapped;
            }
        }
    }
    /* molecules outside the box after wrapping are lost in the reference */
    for (int64_t k = 0; k < s->n; ++k) {
        const double* r = s->r + 3 * k;
        for (int d = 0; d < 3; ++d)
            if (s->cfg.periodic[d] && !(r[d] >= s->bmin[d] && r[d] < s->bmax[d])) return MD_ERR_DEVICE;
    }
    /* DomainDecompBase::populateHaloLayerWithCopies (DomainDecompBase.cpp:317-376) */
    for (int d = 0; d < 3; ++d) {
        if (!s->cfg.periodic[d]) continue;
        const double L = s->bmax[d] - s->bmin[d];
        for (int dir = 0; dir < 2; ++dir) {
            double lo[3], hi[3];
            for (int e = 0; e < 3; ++e) { lo[e] = s->bmin[e] - rc; hi[e] = s->bmax[e] + rc; }
            if (dir == 0) { lo[d] = s->bmin[d]; hi[d] = s->bmin[d] + rc; }
            else { lo[d] = s->bmax[d] - rc; hi[d] = s->bmax[d]; }
            double shift = dir == 0 ? L : -L;
            int64_t end = s->ntot;
            for (int64_t k = 0; k < end; ++k) {
                if (!in_region(s->r + 3 * k, lo, hi)) continue;
                int64_t h = add_copy(s, k);
                double* r = s->r + 3 * h;
                r[d] = r[d] + shift;
                if (shift < 0) {
                    if (r[d] >= s->bmin[d]) r[d] = nextafter(s->bmin[d], -INFINITY);
                } else {
                    if (r[d] < s->bmax[d]) r[d] = nextafter(s->bmax[d], INFINITY);
                }
            }
        }
    }
    /* bin everything (stable counting sort by cell) */
    memset(s->cstart, 0, sizeof(int64_t) * (size_t)(s->ncells + 1));
    int64_t maxocc = 0;
    for (int64_t k = 0; k < s->ntot; ++k) {
        int64_t c = cell_of_point(s, s->r + 3 * k);
        s->mcell[k] = c;
        s->cstart[c + 1]++;
    }
    for (int64_t c = 0; c < s->ncells; ++c) {
        if (s->cstart[c + 1] > maxocc) maxocc = s->cstart[c + 1];
        s->cstart[c + 1] += s->cstart[c];
    }
    {
        int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)s->ncells);
        memcpy(fill, s->cstart, sizeof(int64_t) * (size_t)s->ncells);
        for (int64_t k = 0; k < s->ntot; ++k) s->clist[fill[s->mcell[k]]++] = k;
        free(fill);
    }
    /* FullParticleCell::buildSoACaches -> FullMolecule::setupSoACache
     * (FullParticleCell.cpp:141-190, FullMolecule.cpp:711-767): normalise q,
     * site positions r + R(q) d, orientations R(q) e; clearFM */
    int64_t ns = 0;
    for (int64_t k = 0; k < s->ntot; ++k) {
        s->soff[k] = ns;
        ns += s->cdef[s->mcomp[k]].ns;
    }
    s->soff[s->ntot] = ns;
    if (ns > s->scap) {
        s->scap = ns + 64;
        s->spos = (double*)realloc(s->spos, sizeof(double) * 3 * s->scap);
        s->se = (double*)realloc(s->se, sizeof(double) * 3 * s->scap);
        s->sF = (double*)realloc(s->sF, sizeof(double) * 3 * s->scap);
        s->sV = (double*)realloc(s->sV, sizeof(double) * 3 * s->scap);
        s->sM = (double*)realloc(s->sM, sizeof(double) * 3 * s->scap);
    }
    s->nsites = ns;
    for (int64_t k = 0; k < s->ntot; ++k) {
        double* q = s->q + 4 * k;
        q_normalize(q);
        const ocomp* o = &s->cdef[s->mcomp[k]];
        int64_t b = s->soff[k];
        for (int i = 0; i < o->ns; ++i) {
            const double* dsite;
            const double* esite = NULL;
            if (i < o->nlj) dsite = o->lj[i];
            else if (i < o->nlj + o->nch) dsite = o->ch[i - o->nlj];
            else if (i < o->nlj + o->nch + o->ndi) { dsite = o->di[i - o->nlj - o->nch]; esite = dsite + 3; }
            else { dsite = o->qu[i - o->nlj - o->nch - o->ndi]; esite = dsite + 3; }
            double dr[3];
            q_rotate(q, dsite, dr);
            for (int e = 0; e < 3; ++e) s->spos[3 * (b + i) + e] = dr[e] + s->r[3 * k + e];
            if (esite) q_rotate(q, esite, s->se + 3 * (b + i));
            else s->se[3 * (b + i)] = s->se[3 * (b + i) + 1] = s->se[3 * (b + i) + 2] = 0.0;
        }
    }
    memset(s->sF, 0, sizeof(double) * 3 * ns);
    memset(s->sV, 0, sizeof(double) * 3 * ns);
    memset(s->sM, 0, sizeof(double) * 3 * ns);
    if (st) {
        st->n_inner = s->n;
        st->n_halo = s->ntot - s->n;
        st->max_occupancy = maxocc;
        st->n_wrapped = wrapped;
        for (int d = 0; d < 3; ++d) { st->cells[d] = s->cpd[d]; st->cell_length[d] = s->cl[d]; }
    }
    return MD_OK;
}

int orc_get_cells(const orc_sys* s, int64_t n, int64_t* cell) {
    if (n != s->n) return MD_ERR_ARG;
    for (int64_t k = 0; k < n; ++k) cell[k] = cell_of_point(s, s->r + 3 * k);
    return MD_OK;
}

/* ---------------------------------------------------------------- site-site bodies
 * VectorizedCellProcessor::_loopBody* (VectorizedCellProcessor.cpp:171-792) for
 * the reference's scalar path: fmadd(a,b,c)=a*b+c, fnmadd(a,b,c)=c-a*b,
 * fmsub(a,b,c)=a*b-c, scal_prod(a,b)=a1*b1+(a2*b2+a3*b3) (RealVecDouble.h:159-222),
 * 1/r^2 by division and 1/r = sqrt(1/r^2). */
static inline double sp3(double a1, double a2, double a3, double b1, double b2, double b3) {
    return a1 * b1 + (a2 * b2 + a3 * b3);
}

typedef struct {
    double upot6lj, upotXpoles, virial, myRF;
} macro_t;

/* LJ (VCP.cpp:171-224): f is the force on site 1 */
static void body_lj(const double* m1, const double* r1, const double* m2, const double* r2, double eps24,
                    double sig2, double shift6, int macro, double* f, double* V, macro_t* acc) {
    double dx = r1[0] - r2[0], dy = r1[1] - r2[1], dz = r1[2] - r2[2];
    double r2c = sp3(dx, dy, dz, dx, dy, dz);
    double r2inv = 1.0 / r2c;
    double lj2 = sig2 * r2inv, lj4 = lj2 * lj2, lj6 = lj4 * lj2, lj12 = lj6 * lj6;
    double lj12m6 = lj12 - lj6;
    double eps24r2inv = eps24 * r2inv;
    double lj12lj12m6 = lj12 + lj12m6;
    double scale = eps24r2inv * lj12lj12m6;
    f[0] = dx * scale; f[1] = dy * scale; f[2] = dz * scale;
    double mdx = m1[0] - m2[0], mdy = m1[1] - m2[1], mdz = m1[2] - m2[2];
    V[0] = mdx * f[0]; V[1] = mdy * f[1]; V[2] = mdz * f[2];
    if (macro) {
        double upot = eps24 * lj12m6 + shift6;
        acc->upot6lj = acc->upot6lj + upot;
        acc->virial = acc->virial + V[0] + V[1] + V[2];
    }
}

/* charge-charge (VCP.cpp:227-277) */
static void body_cc(const double* m1, const double* r1, double q1, const double* m2, const double* r2, double q2,
                    int macro, double* f, double* V, macro_t* acc) {
    double dx = r1[0] - r2[0], dy = r1[1] - r2[1], dz = r1[2] - r2[2];
    double dr2 = sp3(dx, dy, dz, dx, dy, dz);
    double dr2inv = 1.0 / dr2;
    double drinv = sqrt(dr2inv);
    double qq = q1 * q2;
    double upot = qq * drinv;
    double fac = upot * dr2inv;
    f[0] = dx * fac; f[1] = dy * fac; f[2] = dz * fac;
    double mdx = m1[0] - m2[0], mdy = m1[1] - m2[1], mdz = m1[2] - m2[2];
    V[0] = mdx * f[0]; V[1] = mdy * f[1]; V[2] = mdz * f[2];
    if (macro) {
        acc->upotXpoles = acc->upotXpoles + upot;
        acc->virial = acc->virial + V[0] + V[1] + V[2];
    }
}

/* charge(1)-dipole(2) (VCP.cpp:279-347): f on the charge, M on the dipole */
static void body_cd(const double* m1, const double* r1, double q, const double* m2, const double* r2,
                    const double* e, double p, int macro, double* f, double* V, double* M, macro_t* acc) {
    double dx = r1[0] - r2[0], dy = r1[1] - r2[1], dz = r1[2] - r2[2];
    double dr2 = sp3(dx, dy, dz, dx, dy, dz);
    double dr2inv = 1.0 / dr2;
    double drinv = sqrt(dr2inv);
    double dr3inv = dr2inv * drinv;
    double re = sp3(dx, dy, dz, e[0], e[1], e[2]);
    double qp = q * p;
    double qpdr3 = qp * dr3inv;
    double fac = dr2inv * 3.0 * re;
    f[0] = qpdr3 * (e[0] - dx * fac);
    f[1] = qpdr3 * (e[1] - dy * fac);
    f[2] = qpdr3 * (e[2] - dz * fac);
    double mdx = m1[0] - m2[0], mdy = m1[1] - m2[1], mdz = m1[2] - m2[2];
    V[0] = mdx * f[0]; V[1] = mdy * f[1]; V[2] = mdz * f[2];
    if (macro) {
        double minusUpot = qpdr3 * re;
        acc->upotXpoles = acc->upotXpoles - minusUpot;
        acc->virial = acc->virial + V[0] + V[1] + V[2];
    }
    double exdy_eydx = e[0] * dy - e[1] * dx;
    double eydz_ezdy = e[1] * dz - e[2] * dy;
    double ezdx_exdz = e[2] * dx - e[0] * dz;
    M[0] = qpdr3 * eydz_ezdy;
    M[1] = qpdr3 * ezdx_exdz;
    M[2] = qpdr3 * exdy_eydx;
}

/* dipole-dipole with reaction field (VCP.cpp:349-442) */
static void body_dd(const double* m1, const double* r1, const double* ei, double pii, const double* m2,
                    const double* r2, const double* ej, double pjj, double epsRFInvrc3, int macro, double* f,
                    double* V, double* M1, double* M2, macro_t* acc) {
    double dx = r1[0] - r2[0], dy = r1[1] - r2[1], dz = r1[2] - r2[2];
    double dr2 = sp3(dx, dy, dz, dx, dy, dz);
    double dr2inv = 1.0 / dr2;
    double drinv = sqrt(dr2inv);
    double dr2three_inv = 3.0 * dr2inv;
    double p1p2 = pii * pjj;
    double rffac = p1p2 * epsRFInvrc3;
    double p1p2r3 = p1p2 * drinv * dr2inv;
    double p1p2threer5 = p1p2r3 * dr2three_inv;
    double e1e2 = sp3(ei[0], ei[1], ei[2], ej[0], ej[1], ej[2]);
    double re1 = sp3(dx, dy, dz, ei[0], ei[1], ei[2]);
    double re2 = sp3(dx, dy, dz, ej[0], ej[1], ej[2]);
    double re1threeperr2 = re1 * dr2three_inv;
    double re2threeperr2 = re2 * dr2three_inv;
    double re1re2perr2 = dr2inv * re1 * re2;
    double e1e2m5 = e1e2 - 5.0 * re1re2perr2;
    f[0] = p1p2threer5 * sp3(dx, ei[0], ej[0], e1e2m5, re2, re1);
    f[1] = p1p2threer5 * sp3(dy, ei[1], ej[1], e1e2m5, re2, re1);
    f[2] = p1p2threer5 * sp3(dz, ei[2], ej[2], e1e2m5, re2, re1);
    double mdx = m1[0] - m2[0], mdy = m1[1] - m2[1], mdz = m1[2] - m2[2];
    V[0] = mdx * f[0]; V[1] = mdy * f[1]; V[2] = mdz * f[2];
    if (macro) {
        double upot = p1p2r3 * (e1e2 - 3.0 * re1re2perr2);
        acc->upotXpoles = acc->upotXpoles + upot;
        acc->virial = acc->virial + V[0] + V[1] + V[2];
        acc->myRF = acc->myRF + rffac * e1e2;
    }
    double e1xe2y = ei[0] * ej[1] - ei[1] * ej[0];
    double e1ye2z = ei[1] * ej[2] - ei[2] * ej[1];
    double e1ze2x = ei[2] * ej[0] - ei[0] * ej[2];
    M1[0] = p1p2r3 * (re2threeperr2 * (ei[1] * dz - ei[2] * dy) - e1ye2z) + rffac * e1ye2z;
    M1[1] = p1p2r3 * (re2threeperr2 * (ei[2] * dx - ei[0] * dz) - e1ze2x) + rffac * e1ze2x;
    M1[2] = p1p2r3 * (re2threeperr2 * (ei[0] * dy - ei[1] * dx) - e1xe2y) + rffac * e1xe2y;
    M2[0] = p1p2r3 * (re1threeperr2 * (ej[1] * dz - ej[2] * dy) + e1ye2z) - rffac * e1ye2z;
    M2[1] = p1p2r3 * (re1threeperr2 * (ej[2] * dx - ej[0] * dz) + e1ze2x) - rffac * e1ze2x;
    M2[2] = p1p2r3 * (re1threeperr2 * (ej[0] * dy - ej[1] * dx) + e1xe2y) - rffac * e1xe2y;
}

/* charge(1)-quadrupole(2) (VCP.cpp:444-524): f on the charge, M on the quadrupole */
static void body_cq(const double* m1, const double* r1, double q, const double* m2, const double* r2,
                    const double* ej, double m, int macro, double* f, double* V, double* M, macro_t* acc) {
    double dx = r1[0] - r2[0], dy = r1[1] - r2[1], dz = r1[2] - r2[2];
    double dr2 = sp3(dx, dy, dz, dx, dy, dz);
    double invdr2 = 1.0 / dr2;
    double invdr = sqrt(invdr2);
    double qQ05 = 0.5 * q * m;
    double costj = sp3(ej[0], ej[1], ej[2], dx, dy, dz);
    costj = costj * invdr;
    double qQinv4dr3 = qQ05 * invdr * invdr2;
    double part1 = 3.0 * costj * costj;
    double upot = qQinv4dr3 * (part1 - 1.0);
    double minus_partialRijInvdr = 3.0 * upot * invdr2;
    double partialTjInvdr = 6.0 * costj * qQinv4dr3 * invdr;
    double fac = costj * partialTjInvdr * invdr + minus_partialRijInvdr;
    f[0] = fac * dx - partialTjInvdr * ej[0];
    f[1] = fac * dy - partialTjInvdr * ej[1];
    f[2] = fac * dz - partialTjInvdr * ej[2];
    double mdx = m1[0] - m2[0], mdy = m1[1] - m2[1], mdz = m1[2] - m2[2];
    V[0] = mdx * f[0]; V[1] = mdy * f[1]; V[2] = mdz * f[2];
    if (macro) {
        acc->upotXpoles = acc->upotXpoles + upot;
        acc->virial = acc->virial + V[0] + V[1] + V[2];
    }
    double mx = ej[2] * dy - ej[1] * dz;
    double my = ej[0] * dz - ej[2] * dx;
    double mz = ej[1] * dx - ej[0] * dy;
    M[0] = partialTjInvdr * mx;
    M[1] = partialTjInvdr * my;
    M[2] = partialTjInvdr * mz;
}

/* dipole(1)-quadrupole(2) (VCP.cpp:526-648) */
static void body_dq(const double* m1, const double* r1, const double* ei, double p, const double* m2,
                    const double* r2, const double* ej, double m, int macro, double* f, double* V, double* M1,
                    double* M2, macro_t* acc) {
    double dx = r1[0] - r2[0], dy = r1[1] - r2[1], dz = r1[2] - r2[2];
    double dr2 = sp3(dx, dy, dz, dx, dy, dz);
    double invdr2 = 1.0 / dr2;
    double invdr = sqrt(invdr2);
    double myqfac = 1.5 * p * m * invdr2 * invdr2;
    double costi = sp3(ei[0], ei[1], ei[2], dx, dy, dz);
    costi = costi * invdr;
    double costj = sp3(ej[0], ej[1], ej[2], dx, dy, dz);
    costj = costj * invdr;
    double cos2tj = costj * costj;
    double cosgij = sp3(ei[0], ei[1], ei[2], ej[0], ej[1], ej[2]);
    double _5cos2tjminus1 = 5.0 * cos2tj - 1.0;
    double _2costj = 2.0 * costj;
    double part1 = costi * _5cos2tjminus1;
    double part2 = _2costj * cosgij;
    double upot = myqfac * (part2 - part1);
    double myqfacXinvdr = myqfac * invdr;
    double minus_partialRijInvdr = 4.0 * upot * invdr2;
    double minus_partialTiInvdr = myqfacXinvdr * _5cos2tjminus1;
    part1 = 5.0 * (costi * costj) - cosgij;
    double minus_partialTjInvdr = myqfacXinvdr * 2.0 * part1;
    double partialGij = myqfac * _2costj;
    double part3 = costi * minus_partialTiInvdr + costj * minus_partialTjInvdr;
    double fac = minus_partialRijInvdr - part3 * invdr;
    f[0] = sp3(fac, minus_partialTiInvdr, minus_partialTjInvdr, dx, ei[0], ej[0]);
    f[1] = sp3(fac, minus_partialTiInvdr, minus_partialTjInvdr, dy, ei[1], ej[1]);
    f[2] = sp3(fac, minus_partialTiInvdr, minus_partialTjInvdr, dz, ei[2], ej[2]);
    double mdx = m1[0] - m2[0], mdy = m1[1] - m2[1], mdz = m1[2] - m2[2];
    V[0] = mdx * f[0]; V[1] = mdy * f[1]; V[2] = mdz * f[2];
    if (macro) {
        acc->upotXpoles = acc->upotXpoles + upot;
        acc->virial = acc->virial + V[0] + V[1] + V[2];
    }
    double eixejy = ei[0] * ej[1] - ei[1] * ej[0];
    double eiyejz = ei[1] * ej[2] - ei[2] * ej[1];
    double eizejx = ei[2] * ej[0] - ei[0] * ej[2];
    double gx = partialGij * eiyejz, gy = partialGij * eizejx, gz = partialGij * eixejy;
    double ax = ei[1] * dz - ei[2] * dy, ay = ei[2] * dx - ei[0] * dz, az = ei[0] * dy - ei[1] * dx;
    M1[0] = minus_partialTiInvdr * ax - gx;
    M1[1] = minus_partialTiInvdr * ay - gy;
    M1[2] = minus_partialTiInvdr * az - gz;
    double bx = ej[1] * dz - ej[2] * dy, by = ej[2] * dx - ej[0] * dz, bz = ej[0] * dy - ej[1] * dx;
    M2[0] = minus_partialTjInvdr * bx + gx;
    M2[1] = minus_partialTjInvdr * by + gy;
    M2[2] = minus_partialTjInvdr * bz + gz;
}

/* quadrupole-quadrupole (VCP.cpp:650-792) */
static void body_qq(const double* m1, const double* r1, const double* ei, double mii, const double* m2,
                    const double* r2, const double* ej, double mjj, int macro, double* f, double* V, double* M1,
                    double* M2, macro_t* acc) {
    double dx = r1[0] - r2[0], dy = r1[1] - r2[1], dz = r1[2] - r2[2];
    double dr2 = sp3(dx, dy, dz, dx, dy, dz);
    double invdr2 = 1.0 / dr2;
    double invdr = sqrt(invdr2);
    double qfac = 0.75 * invdr;
    qfac = qfac * (mii * mjj);
    qfac = qfac * (invdr2 * invdr2);
    double costi = sp3(ei[0], ei[1], ei[2], dx, dy, dz);
    costi = costi * invdr;
    double costj = sp3(ej[0], ej[1], ej[2], dx, dy, dz);
    costj = costj * invdr;
    double cos2ti = costi * costi, cos2tj = costj * costj;
    double cosgij = sp3(ei[0], ei[1], ei[2], ej[0], ej[1], ej[2]);
    double term = 5.0 * (costi * costj);
    term = cosgij - term;
    double part2 = 15.0 * cos2ti * cos2tj;
    double part3 = 2.0 * term * term;
    double upot = 5.0 * (cos2ti + cos2tj) + part2;
    upot = (1.0 + part3) - upot;
    upot = qfac * upot;
    double minus_partialRijInvdr = 5.0 * upot * invdr2;
    double part1 = qfac * 10.0 * invdr;
    part2 = 2.0 * term;
    part3 = 3.0 * costi * cos2tj;
    double part4 = costi + (part2 * costj + part3);
    double minus_partialTiInvdr = part1 * part4;
    part3 = 3.0 * costj * cos2ti;
    part4 = costj + (part2 * costi + part3);
    double minus_partialTjInvdr = part1 * part4;
    double partialGij = qfac * 4.0 * term;
    part1 = minus_partialTiInvdr * costi;
    part2 = minus_partialTjInvdr * costj;
    double fac = minus_partialRijInvdr - (part1 + part2) * invdr;
    f[0] = sp3(fac, minus_partialTiInvdr, minus_partialTjInvdr, dx, ei[0], ej[0]);
    f[1] = sp3(fac, minus_partialTiInvdr, minus_partialTjInvdr, dy, ei[1], ej[1]);
    f[2] = sp3(fac, minus_partialTiInvdr, minus_partialTjInvdr, dz, ei[2], ej[2]);
    double mdx = m1[0] - m2[0], mdy = m1[1] - m2[1], mdz = m1[2] - m2[2];
    V[0] = mdx * f[0]; V[1] = mdy * f[1]; V[2] = mdz * f[2];
    if (macro) {
        acc->upotXpoles = acc->upotXpoles + upot;
        acc->virial = acc->virial + V[0] + V[1] + V[2];
    }
    double eixejy = ei[0] * ej[1] - ei[1] * ej[0];
    double eiyejz = ei[1] * ej[2] - ei[2] * ej[1];
    double eizejx = ei[2] * ej[0] - ei[0] * ej[2];
    double gx = partialGij * eiyejz, gy = partialGij * eizejx, gz = partialGij * eixejy;
    double ax = ei[1] * dz - ei[2] * dy, ay = ei[2] * dx - ei[0] * dz, az = ei[0] * dy - ei[1] * dx;
    M1[0] = minus_partialTiInvdr * ax - gx;
    M1[1] = minus_partialTiInvdr * ay - gy;
    M1[2] = minus_partialTiInvdr * az - gz;
    double bx = ej[1] * dz - ej[2] * dy, by = ej[2] * dx - ej[0] * dz, bz = ej[0] * dy - ej[1] * dx;
    M2[0] = minus_partialTjInvdr * bx + gx;
    M2[1] = minus_partialTjInvdr * by + gy;
    M2[2] = minus_partialTjInvdr * bz + gz;
}

/* ---------------------------------------------------------------- pair driver
 * One (molecule a of soa1, molecule b of soa2) pair, all site combinations in
 * the order of VCP::_calculatePairs (VCP.cpp:794-2730): the i-side sums are
 * accumulated in isum[] and stored after the j loop by the caller. */
typedef struct {
    double kcalls[8]; /* molecule distances + 7 kinds (all visits) */
    double mcalls[8]; /* macroscopic only */
    macro_t acc;
} tstate;

static inline void add3(double* a, const double* b) { a[0] += b[0]; a[1] += b[1]; a[2] += b[2]; }
static inline void sub3(double* a, const double* b) { a[0] -= b[0]; a[1] -= b[1]; a[2] -= b[2]; }

/* i-side partial sums of one molecule a against all molecules of a cell */
typedef struct {
    double F[MAXS * 4][3], V[MAXS * 4][3], M[MAXS * 4][3];
} iside;

static void pair_molecules(orc_sys* s, int64_t a, int64_t b, int macro, iside* is, tstate* ts, double rcLJ2,
                           double rc2, int single) {
    const double* ra = s->r + 3 * a;
    const double* rb = s->r + 3 * b;
    double mdx = ra[0] - rb[0], mdy = ra[1] - rb[1], mdz = ra[2] - rb[2];
    double mr2 = sp3(mdx, mdy, mdz, mdx, mdy, mdz);
    if (single && mr2 == 0.0) return;
    const ocomp* A = &s->cdef[s->mcomp[a]];
    const ocomp* B = &s->cdef[s->mcomp[b]];
    const int64_t sa = s->soff[a], sb = s->soff[b];
    double* P = s->spos;
    double* E = s->se;
    double f[3], V[3], M1[3], M2[3];
    const int lj_on = mr2 < rcLJ2, el_on = mr2 < rc2;
    ts->kcalls[0] += 1;
    if (lj_on) {
        ts->kcalls[1] += A->nlj * B->nlj;
        if (macro) ts->mcalls[1] += A->nlj * B->nlj;
        for (int i = 0; i < A->nlj; ++i)
            for (int j = 0; j < B->nlj; ++j) {
                int gi = A->ljoff + i, gj = B->ljoff + j;
                body_lj(ra, P + 3 * (sa + i), rb, P + 3 * (sb + j), s->eps24[gi * s->nlj + gj], s->sig2[gi * s->nlj + gj],
                        s->shift6[gi * s->nlj + gj], macro, f, V, &ts->acc);
                sub3(s->sF + 3 * (sb + j), f);
                add3(s->sV + 3 * (sb + j), V);
                add3(is->F[i], f);
                add3(is->V[i], V);
            }
    }
    if (!el_on) return;
    const int ac = A->nlj, ad = ac + A->nch, aq = ad + A->ndi;
    const int bc = B->nlj, bd = bc + B->nch, bq = bd + B->ndi;
    ts->kcalls[2] += A->nch * B->nch;
    ts->kcalls[3] += A->nch * B->ndi + A->ndi * B->nch;
    ts->kcalls[4] += A->ndi * B->ndi;
    ts->kcalls[5] += A->nch * B->nqu + A->nqu * B->nch;
    ts->kcalls[6] += A->ndi * B->nqu + A->nqu * B->ndi;
    ts->kcalls[7] += A->nqu * B->nqu;
    if (macro) {
        ts->mcalls[0] += 1;
        ts->mcalls[2] += A->nch * B->nch;
        ts->mcalls[3] += A->nch * B->ndi + A->ndi * B->nch;
        ts->mcalls[4] += A->ndi * B->ndi;
        ts->mcalls[5] += A->nch * B->nqu + A->nqu * B->nch;
        ts->mcalls[6] += A->ndi * B->nqu + A->nqu * B->ndi;
        ts->mcalls[7] += A->nqu * B->nqu;
    }
    /* charges of a: vs charges, dipoles, quadrupoles of b */
    for (int i = 0; i < A->nch; ++i) {
        const double* ri = P + 3 * (sa + ac + i);
        double qi = A->ch[i][4];
        for (int j = 0; j < B->nch; ++j) {
            body_cc(ra, ri, qi, rb, P + 3 * (sb + bc + j), B->ch[j][4], macro, f, V, &ts->acc);
            sub3(s->sF + 3 * (sb + bc + j), f); add3(s->sV + 3 * (sb + bc + j), V);
            add3(is->F[ac + i], f); add3(is->V[ac + i], V);
        }
        for (int j = 0; j < B->ndi; ++j) {
            int64_t js = sb + bd + j;
            body_cd(ra, ri, qi, rb, P + 3 * js, E + 3 * js, B->di[j][6], macro, f, V, M1, &ts->acc);
            sub3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V); add3(s->sM + 3 * js, M1);
            add3(is->F[ac + i], f); add3(is->V[ac + i], V);
        }
        for (int j = 0; j < B->nqu; ++j) {
            int64_t js = sb + bq + j;
            body_cq(ra, ri, qi, rb, P + 3 * js, E + 3 * js, B->qu[j][6], macro, f, V, M1, &ts->acc);
            sub3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V); add3(s->sM + 3 * js, M1);
            add3(is->F[ac + i], f); add3(is->V[ac + i], V);
        }
    }
    /* dipoles of a */
    for (int i = 0; i < A->ndi; ++i) {
        int64_t is_ = sa + ad + i;
        const double* ri = P + 3 * is_;
        const double* ei = E + 3 * is_;
        double pi = A->di[i][6];
        for (int j = 0; j < B->ndi; ++j) {
            int64_t js = sb + bd + j;
            body_dd(ra, ri, ei, pi, rb, P + 3 * js, E + 3 * js, B->di[j][6], s->epsRFInvrc3, macro, f, V, M1, M2,
                    &ts->acc);
            sub3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V); add3(s->sM + 3 * js, M2);
            add3(is->F[ad + i], f); add3(is->V[ad + i], V); add3(is->M[ad + i], M1);
        }
        for (int j = 0; j < B->nch; ++j) {  /* charge of b is site 1 */
            int64_t js = sb + bc + j;
            body_cd(rb, P + 3 * js, B->ch[j][4], ra, ri, ei, pi, macro, f, V, M1, &ts->acc);
            add3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V);
            sub3(is->F[ad + i], f); add3(is->V[ad + i], V); add3(is->M[ad + i], M1);
        }
        for (int j = 0; j < B->nqu; ++j) {
            int64_t js = sb + bq + j;
            body_dq(ra, ri, ei, pi, rb, P + 3 * js, E + 3 * js, B->qu[j][6], macro, f, V, M1, M2, &ts->acc);
            sub3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V); add3(s->sM + 3 * js, M2);
            add3(is->F[ad + i], f); add3(is->V[ad + i], V); add3(is->M[ad + i], M1);
        }
    }
    /* quadrupoles of a */
    for (int i = 0; i < A->nqu; ++i) {
        int64_t is_ = sa + aq + i;
        const double* ri = P + 3 * is_;
        const double* ei = E + 3 * is_;
        double mi = A->qu[i][6];
        for (int j = 0; j < B->nqu; ++j) {
            int64_t js = sb + bq + j;
            body_qq(ra, ri, ei, mi, rb, P + 3 * js, E + 3 * js, B->qu[j][6], macro, f, V, M1, M2, &ts->acc);
            sub3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V); add3(s->sM + 3 * js, M2);
            add3(is->F[aq + i], f); add3(is->V[aq + i], V); add3(is->M[aq + i], M1);
        }
        for (int j = 0; j < B->nch; ++j) {  /* charge of b is site 1 */
            int64_t js = sb + bc + j;
            body_cq(rb, P + 3 * js, B->ch[j][4], ra, ri, ei, mi, macro, f, V, M1, &ts->acc);
            add3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V);
            sub3(is->F[aq + i], f); add3(is->V[aq + i], V); add3(is->M[aq + i], M1);
        }
        for (int j = 0; j < B->ndi; ++j) {  /* dipole of b is site 1 */
            int64_t js = sb + bd + j;
            body_dq(rb, P + 3 * js, E + 3 * js, B->di[j][6], ra, ri, ei, mi, macro, f, V, M1, M2, &ts->acc);
            add3(s->sF + 3 * js, f); add3(s->sV + 3 * js, V); add3(s->sM + 3 * js, M1);
            sub3(is->F[aq + i], f); add3(is->V[aq + i], V); add3(is->M[aq + i], M2);
        }
    }
}

/* VCP::_calculatePairs over soa1 x soa2 (single: same cell, j after i) */
static void calc_pairs(orc_sys* s, int64_t c1, int64_t c2, int macro, int single, tstate* ts) {
    const double rcLJ2 = s->cfg.rc_lj * s->cfg.rc_lj, rc2 = s->cfg.rc * s->cfg.rc;
    iside is;
    macro_t saved = ts->acc;
    macro_t local = {0, 0, 0, 0};
    ts->acc = local;
    for (int64_t x = s->cstart[c1]; x < s->cstart[c1 + 1]; ++x) {
        int64_t a = s->clist[x];
        const ocomp* A = &s->cdef[s->mcomp[a]];
        for (int i = 0; i < A->ns; ++i)
            for (int e = 0; e < 3; ++e) is.F[i][e] = is.V[i][e] = is.M[i][e] = 0.0;
        int64_t y0 = single ? x + 1 : s->cstart[c2];
        for (int64_t y = y0; y < s->cstart[c2 + 1]; ++y) pair_molecules(s, a, s->clist[y], macro, &is, ts, rcLJ2, rc2, single);
        int64_t sa = s->soff[a];
        for (int i = 0; i < A->ns; ++i) {
            add3(s->sF + 3 * (sa + i), is.F[i]);
            add3(s->sV + 3 * (sa + i), is.V[i]);
            add3(s->sM + 3 * (sa + i), is.M[i]);
        }
    }
    /* per-call totals are added to the thread accumulators (VCP.cpp:2723-2728) */
    saved.upot6lj += ts->acc.upot6lj;
    saved.upotXpoles += ts->acc.upotXpoles;
    saved.virial += ts->acc.virial;
    saved.myRF += 0.0 - ts->acc.myRF;
    ts->acc = saved;
}

static int is_halo_cell(const orc_sys* s, int64_t c) {
    int x = (int)(c % s->cpd[0]), y = (int)((c / s->cpd[0]) % s->cpd[1]), z = (int)(c / ((int64_t)s->cpd[0] * s->cpd[1]));
    return x == 0 || y == 0 || z == 0 || x == s->cpd[0] - 1 || y == s->cpd[1] - 1 || z == s->cpd[2] - 1;
}

/* VCP::processCell / processCellPair (VCP.cpp:2732-2819) */
static void process_cell(orc_sys* s, int64_t c, tstate* ts) {
    if (is_halo_cell(s, c) || s->cstart[c + 1] - s->cstart[c] < 2) return;
    calc_pairs(s, c, c, 1, 1, ts);
}

static void process_cell_pair(orc_sys* s, int64_t c1, int64_t c2, tstate* ts) {
    int64_t n1 = s->cstart[c1 + 1] - s->cstart[c1], n2 = s->cstart[c2 + 1] - s->cstart[c2];
    if (n1 == 0 || n2 == 0) return;
    int h1 = is_halo_cell(s, c1), h2 = is_halo_cell(s, c2);
    if (h1 && h2) return;
    int macro = (!h1 && !h2) || (c1 < c2);
    if (n1 <= n2) calc_pairs(s, c1, c2, macro, 0, ts);
    else calc_pairs(s, c2, c1, macro, 0, ts);
}

/* C08BasedTraversals::processBaseCell (C08BasedTraversals.h:48-100, offsets :102-152) */
static void process_base_cell(orc_sys* s, int64_t base, const int64_t off[14][2], tstate* ts) {
    for (int j = 0; j < 14; ++j) {
        int64_t c1 = base + off[j][0], c2 = base + off[j][1];
        if (is_halo_cell(s, c1) && is_halo_cell(s, c2)) continue;
        if (c1 == c2) process_cell(s, c1, ts);
        else if (!is_halo_cell(s, c1)) process_cell_pair(s, c1, c2, ts);
        else process_cell_pair(s, c2, c1, ts);
    }
}

int orc_forces(orc_sys* s, md_forces_out* out, double* kernel_calls) {
    const int64_t X = s->cpd[0], Y = s->cpd[1], Z = s->cpd[2];
    const int64_t o = 0, x = 1, y = X, z = X * Y, xy = x + y, yz = y + z, xz = x + z, xyz = x + y + z;
    const int64_t off[14][2] = {{o, o}, {o, y}, {y, z}, {o, z}, {o, yz}, {x, yz}, {x, y},
                                {x, z}, {o, x}, {o, xy}, {xy, z}, {y, xz}, {o, xz}, {o, xyz}};
    int nthr = g_threads;
    tstate* ts = (tstate*)calloc((size_t)nthr, sizeof(tstate));
    /* C08CellPairTraversal::traverseCellPairs (C08CellPairTraversal.h:46-75, 197-231) */
    for (int col = 0; col < 8; ++col) {
        int64_t sx = col & 1, sy = (col >> 1) & 1, sz = (col >> 2) & 1;
        int64_t nbx = (X - 1 - sx + 1) / 2, nby = (Y - 1 - sy + 1) / 2, nbz = (Z - 1 - sz + 1) / 2;
        int64_t nb = nbx * nby * nbz;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 4)
#endif
        for (int64_t t = 0; t < nb; ++t) {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            int64_t bx = sx + 2 * (t % nbx), by = sy + 2 * ((t / nbx) % nby), bz = sz + 2 * (t / (nbx * nby));
            process_base_cell(s, (bz * Y + by) * X + bx, off, &ts[tid]);
        }
    }
    macro_t tot = {0, 0, 0, 0};
    double kc[8] = {0}, mc[8] = {0};
    for (int t = 0; t < nthr; ++t) {
        tot.upot6lj += ts[t].acc.upot6lj;
        tot.upotXpoles += ts[t].acc.upotXpoles;
        tot.virial += ts[t].acc.virial;
        tot.myRF += ts[t].acc.myRF;
        for (int k = 0; k < 8; ++k) { kc[k] += ts[t].kcalls[k]; mc[k] += ts[t].mcalls[k]; }
    }
    free(ts);
    /* FullMolecule::calcFM (FullMolecule.cpp:523-631) for the inner molecules */
    for (int64_t k = 0; k < s->n; ++k) {
        const ocomp* C = &s->cdef[s->mcomp[k]];
        const double* q = s->q + 4 * k;
        double* F = s->F + 3 * k;
        double* M = s->M + 3 * k;
        double* Vi = s->Vi + 3 * k;
        F[0] = F[1] = F[2] = 0.; M[0] = M[1] = M[2] = 0.; Vi[0] = Vi[1] = Vi[2] = 0.;
        double tM[3] = {0, 0, 0}, tV[3] = {0, 0, 0};
        int64_t b = s->soff[k];
        for (int i = 0; i < C->ns; ++i) {
            const double* dsrc;
            if (i < C->nlj) dsrc = C->lj[i];
            else if (i < C->nlj + C->nch) dsrc = C->ch[i - C->nlj];
            else if (i < C->nlj + C->nch + C->ndi) dsrc = C->di[i - C->nlj - C->nch];
            else dsrc = C->qu[i - C->nlj - C->nch - C->ndi];
            double ds[3];
            q_rotate(q, dsrc, ds);
            const double* Fs = s->sF + 3 * (b + i);
            F[0] += Fs[0]; F[1] += Fs[1]; F[2] += Fs[2];
            M[0] += ds[1] * Fs[2] - ds[2] * Fs[1];
            M[1] += ds[2] * Fs[0] - ds[0] * Fs[2];
            M[2] += ds[0] * Fs[1] - ds[1] * Fs[0];
            const double* Vs = s->sV + 3 * (b + i);
            tV[0] += Vs[0]; tV[1] += Vs[1]; tV[2] += Vs[2];
            if (i >= C->nlj + C->nch) {
                const double* Ms = s->sM + 3 * (b + i);
                tM[0] += Ms[0]; tM[1] += Ms[1]; tM[2] += Ms[2];
            }
        }
        tV[0] *= 0.5; tV[1] *= 0.5; tV[2] *= 0.5;
        Vi[0] += tV[0]; Vi[1] += tV[1]; Vi[2] += tV[2];
        M[0] += tM[0]; M[1] += tM[1]; M[2] += tM[2];
    }
    /* VCP::endTraversal (VCP.cpp:122-155) */
    if (out) {
        out->upot6lj = tot.upot6lj;
        out->upot_xpoles = tot.upotXpoles;
        out->virial_pairs = tot.virial;
        out->my_rf = tot.myRF;
        out->virial = tot.virial + 3.0 * tot.myRF;
        out->upot = tot.upot6lj / 6.0 + tot.upotXpoles + tot.myRF;
        out->mol_pairs = (int64_t)mc[0];
        for (int k = 0; k < MD_NUM_KINDS; ++k) out->site_pairs[k] = (int64_t)mc[k + 1];
    }
    if (kernel_calls)
        for (int k = 0; k < 8; ++k) kernel_calls[k] = kc[k];
    return MD_OK;
}

/* ---------------------------------------------------------------- Leapfrog
 * FullMolecule::upd_preF (FullMolecule.cpp:331-361) */
int orc_pre(orc_sys* s, double dt) {
    for (int64_t k = 0; k < s->n; ++k) {
        const ocomp* C = &s->cdef[s->mcomp[k]];
        double* r = s->r + 3 * k;
        double* v = s->v + 3 * k;
        double* q = s->q + 4 * k;
        double* L = s->L + 3 * k;
        const double* F = s->F + 3 * k;
        const double* M = s->M + 3 * k;
        double dt_halve = .5 * dt;
        double dtInv2m = dt_halve / C->m;
        for (int d = 0; d < 3; ++d) {
            v[d] += dtInv2m * F[d];
            r[d] += dt * v[d];
        }
        double w[3];
        q_rotateinv(q, L, w);
        for (int d = 0; d < 3; ++d) w[d] *= C->invI[d];
        double qh[4];
        q_differentiate(q, w, qh);
        q_scale(qh, dt_halve);
        for (int e = 0; e < 4; ++e) qh[e] += q[e];
        double qcorr = 1. / sqrt(q_mag2(qh));
        q_scale(qh, qcorr);
        for (int d = 0; d < 3; ++d) L[d] += dt_halve * M[d];
        q_rotateinv(qh, L, w);
        for (int d = 0; d < 3; ++d) w[d] *= C->invI[d];
        double qi[4];
        q_differentiate(qh, w, qi);
        q_scale(qi, dt);
        for (int e = 0; e < 4; ++e) q[e] += qi[e];
        qcorr = 1. / sqrt(q_mag2(q));
        q_scale(q, qcorr);
    }
    return MD_OK;
}

/* FullMolecule::upd_postF + Leapfrog::transition2to3 (FullMolecule.cpp:363-389, Leapfrog.cpp:63-147) */
int orc_post(orc_sys* s, double dt, md_kinetic_out* out) {
    double summv2 = 0.0, sumIw2 = 0.0;
    int64_t rot = 0;
    double dt_halve = 0.5 * dt;
    for (int64_t k = 0; k < s->n; ++k) {
        const ocomp* C = &s->cdef[s->mcomp[k]];
        double* v = s->v + 3 * k;
        double* L = s->L + 3 * k;
        const double* F = s->F + 3 * k;
        const double* M = s->M + 3 * k;
        double dtInv2m = dt_halve / C->m;
        double v2 = 0.;
        for (int d = 0; d < 3; ++d) {
            v[d] += dtInv2m * F[d];
            v2 += v[d] * v[d];
            L[d] += dt_halve * M[d];
        }
        summv2 += C->m * v2;
        double w[3];
        q_rotateinv(s->q + 4 * k, L, w);
        double Iw2 = 0.;
        for (int d = 0; d < 3; ++d) {
            w[d] *= C->invI[d];
            Iw2 += C->I[d] * w[d] * w[d];
        }
        sumIw2 += Iw2;
        rot += C->rot_dof;
    }
    if (out) {
        out->summv2 = summv2;
        out->sumIw2 = sumIw2;
        out->n = s->n;
        out->rot_dof = rot;
    }
    return MD_OK;
}

int orc_set_thermostat(orc_sys* s, double target_temperature, int32_t explosion_heuristics) {
    s->thermo_T = target_temperature;
    s->thermo_heur = explosion_heuristics != 0;
    s->th_counter = s->th_warning = s->th_error = 0;
    return MD_OK;
}

/* One global thermostat: Domain::calculateGlobalValues (Domain.cpp:212-345;
 * beta_trans = (3 N T / sum m v^2)^0.4, beta_rot = (rotDOF T / sum I w^2)^0.4,
 * and the explosion heuristic: when a beta falls below MIN_BETA = 0.9,
 * molecules above 10 T of translational (3 rotDOF T of rotational) kinetic
 * energy are slowed down to it, the betas become 1 and beta_rot^0.0091, and
 * the counters advance), then VelocityScalingThermostat::apply
 * (VelocityScalingThermostat.cpp:67-96): v *= beta_trans, D *= beta_rot. */
int orc_thermostat(orc_sys* s, const md_kinetic_out* ko, double* beta_trans, double* beta_rot) {
    const double Ti = s->thermo_T;
    const unsigned long N = (unsigned long)ko->n, rotDOF = (unsigned long)ko->rot_dof;
    const double summv2 = ko->summv2, sumIw2 = rotDOF > 0 ? ko->sumIw2 : 0.0;
    double bt = 1.0, br = 1.0;
    if (Ti > 0.0 && N > 0) {
        bt = pow(3.0 * N * Ti / summv2, 0.4);
        br = sumIw2 == 0.0 ? 1.0 : pow(rotDOF * Ti / sumIw2, 0.4);
    }
    if ((bt < 0.9 || br < 0.9) && 0 >= s->th_error && s->thermo_heur) {
        const double limit_energy = 10.0 * Ti;
        for (int64_t k = 0; k < s->n; ++k) {
            const ocomp* C = &s->cdef[s->mcomp[k]];
            double* v = s->v + 3 * k;
            const double ut = 0.5 * C->m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (ut > limit_energy) {
                const double c = sqrt(limit_energy / ut);
                for (int d = 0; d < 3; ++d) { v[d] *= c; s->F[3 * k + d] *= c; }
            }
            if (C->rot_dof > 0) {
                const double limit_rot = 3.0 * C->rot_dof * Ti;
                double w[3];
                q_rotateinv(s->q + 4 * k, s->L + 3 * k, w);
                double Iw2 = 0.;
                for (int d = 0; d < 3; ++d) {
                    w[d] *= C->invI[d];
                    Iw2 += C->I[d] * w[d] * w[d];
                }
                const double ur = 0.5 * Iw2;
                if (ur > limit_rot) {
                    const double c = sqrt(limit_rot / ur);
                    for (int d = 0; d < 3; ++d) { s->L[3 * k + d] *= c; s->M[3 * k + d] *= c; }
                }
            }
        }
        const int since = 4000 - s->th_counter;
        if (since >= 40) {
            if (s->th_warning > 0) s->th_error = s->th_warning;
            if (s->th_counter > 0) s->th_warning = s->th_counter;
            s->th_counter = 4000;
        }
        bt = 1.0;
        br = pow(br, 0.0091);
    }
    if (s->th_counter > 0) s->th_counter--;
    if (s->th_warning > 0) s->th_warning--;
    if (s->th_error > 0) s->th_error--;
    for (int64_t k = 0; k < s->n; ++k)
        for (int d = 0; d < 3; ++d) {
            s->v[3 * k + d] *= bt;
            s->L[3 * k + d] *= br;
        }
    if (beta_trans) *beta_trans = bt;
    if (beta_rot) *beta_rot = br;
    return MD_OK;
}

/* Simulation::simulateOneTimestep hot part (Simulation.cpp:1076-1300): NVE, or
 * with the global velocity-scaling thermostat after the global values. */
int orc_run(orc_sys* s, double dt, int32_t nsteps, md_step_record* rec) {
    for (int32_t k = 0; k < nsteps; ++k) {
        orc_pre(s, dt);
        int rc = orc_rebin_and_halo(s, NULL);
        if (rc) return rc;
        md_forces_out fo;
        orc_forces(s, &fo, NULL);
        md_kinetic_out ko;
        orc_post(s, dt, &ko);
        if (rec) {
            rec[k].upot = fo.upot;
            rec[k].virial = fo.virial;
            rec[k].summv2 = ko.summv2;
            rec[k].sumIw2 = ko.rot_dof > 0 ? ko.sumIw2 : 0.0;
        }
        if (s->thermo_T > 0.0) orc_thermostat(s, &ko, NULL, NULL);
    }
    return MD_OK;
}

/* ---------------------------------------------------------------- reduced memory mode
 * VCP1CLJRMM (VCP1CLJRMM.cpp:240-369) computes the single-centre LJ pairs of
 * the same traversal and adds dt_inv_m times each pair force to the two
 * velocities at once instead of storing forces; here the traversal's forces
 * are summed first and added once per molecule (the same sum in another
 * order).  Upot = upot6lj / 6 and the virial as in VCP::endTraversal. */
int orc_rmm_forces(orc_sys* s, double dt_inv_m, md_forces_out* out) {
    int rc = orc_rebin_and_halo(s, NULL);
    if (rc) return rc;
    orc_forces(s, out, NULL);
    for (int64_t k = 0; k < 3 * s->n; ++k) s->v[k] += dt_inv_m * s->F[k];
    return MD_OK;
}

/* PositionCellProcessorRMM::processCell (PositionCellProcessorRMM.h:33-60) */
int orc_rmm_positions(orc_sys* s, double dt) {
    for (int64_t k = 0; k < 3 * s->n; ++k) s->r[k] += dt * s->v[k];
    return MD_OK;
}

/* VelocityCellProcessorRMM::processCell (VelocityCellProcessorRMM.h:95-128):
 * sum of v.v, no mass; LeapfrogRMM::computeVelocities reports it with
 * sumIw2 = 0 and no rotational degrees of freedom (LeapfrogRMM.cpp:97-105). */
int orc_rmm_velocities(const orc_sys* s, md_kinetic_out* out) {
    double sum = 0.0;
    for (int64_t k = 0; k < s->n; ++k) {
        const double* v = s->v + 3 * k;
        sum += v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    }
    if (out) {
        out->summv2 = sum;
        out->sumIw2 = 0.0;
        out->n = s->n;
        out->rot_dof = 0;
    }
    return MD_OK;
}

/* One LeapfrogRMM step per iteration: eventNewTimestep (positions), the
 * container update, the force traversal with dt_inv_m = dt / m
 * (VCP1CLJRMM.cpp:41-44), eventForcesCalculated (velocity sums). */
int orc_rmm_run(orc_sys* s, double dt, int32_t nsteps, md_step_record* rec) {
    const double dt_inv_m = dt / s->cdef[0].m;
    for (int32_t k = 0; k < nsteps; ++k) {
        orc_rmm_positions(s, dt);
        md_forces_out fo;
        int rc = orc_rmm_forces(s, dt_inv_m, &fo);
        if (rc) return rc;
        md_kinetic_out ko;
        orc_rmm_velocities(s, &ko);
        if (rec) {
            rec[k].upot = fo.upot;
            rec[k].virial = fo.virial;
            rec[k].summv2 = ko.summv2;
            rec[k].sumIw2 = 0.0;
        }
    }
    return MD_OK;
}

/* ---------------------------------------------------------------- long range
 * Homogeneous::init + calculateLongRange (src/longRange/Homogeneous.cpp:22-146)
 * with its tail integrals (Homogeneous.cpp:158-196): for every pair of LJ
 * centres whose shift6 is zero, the integral of the LJ potential (virial)
 * beyond rcLJ over a uniform fluid, in the form for two centred sites, one
 * centred and one off-centre site (distance tau from its molecule's centre),
 * or two off-centre sites; weighted with N_i N_j eps24 and scaled by
 * pi rho / (3 N).  Plus the reaction-field self term of each component's net
 * dipole (sum of q r over its charges and of the unit-normalised point
 * dipoles), -1/2 epsRFInvrc3 sum_i N_i |mu_i|^2, counted once in Upot and
 * three times in the virial.  The operation order is the reference's. */
static double tl_cc_u(int n, double rc, double s2) {
    return -pow(rc, 2 * n + 3) / (pow(s2, n) * (2 * n + 3));
}
static double tl_cs_u(int n, double rc, double s2, double t) {
    return -(pow(rc + t, 2 * n + 3) - pow(rc - t, 2 * n + 3)) * rc / (4 * pow(s2, n) * t * (n + 1) * (2 * n + 3)) +
           (pow(rc + t, 2 * n + 4) - pow(rc - t, 2 * n + 4)) / (4 * pow(s2, n) * t * (n + 1) * (2 * n + 3) * (2 * n + 4));
}
static double tl_ss_u(int n, double rc, double s2, double t1, double t2) {
    double tp = t1 + t2, tm = t1 - t2;
    return -(pow(rc + tp, 2 * n + 4) - pow(rc + tm, 2 * n + 4) - pow(rc - tm, 2 * n + 4) + pow(rc - tp, 2 * n + 4)) *
               rc / (8 * pow(s2, n) * t1 * t2 * (n + 1) * (2 * n + 3) * (2 * n + 4)) +
           (pow(rc + tp, 2 * n + 5) - pow(rc + tm, 2 * n + 5) - pow(rc - tm, 2 * n + 5) + pow(rc - tp, 2 * n + 5)) /
               (8 * pow(s2, n) * t1 * t2 * (n + 1) * (2 * n + 3) * (2 * n + 4) * (2 * n + 5));
}
static double tl_cc_v(int n, double rc, double s2) { return 2 * n * tl_cc_u(n, rc, s2); }
static double tl_cs_v(int n, double rc, double s2, double t) {
    return -(pow(rc + t, 2 * n + 2) - pow(rc - t, 2 * n + 2)) * rc * rc / (4 * pow(s2, n) * t * (n + 1)) -
           3 * tl_cs_u(n, rc, s2, t);
}
static double tl_ss_v(int n, double rc, double s2, double t1, double t2) {
    double tp = t1 + t2, tm = t1 - t2;
    return -(pow(rc + tp, 2 * n + 3) - pow(rc + tm, 2 * n + 3) - pow(rc - tm, 2 * n + 3) + pow(rc - tp, 2 * n + 3)) *
               rc * rc / (8 * pow(s2, n) * t1 * t2 * (n + 1) * (2 * n + 3)) -
           3 * tl_ss_u(n, rc, s2, t1, t2);
}

int orc_longrange_homogeneous(const orc_sys* s, double* upot_corr, double* virial_corr) {
    const double rclj = s->cfg.rc_lj, rc = s->cfg.rc;
    double cnt[MAXC] = {0};
    for (int64_t k = 0; k < s->n; ++k) cnt[s->mcomp[k]] += 1.0;
    double U = 0.0, W = 0.0, self = 0.0;
    unsigned long nmol = 0;
    for (int i = 0; i < s->ncomp; ++i) {
        const ocomp* ci = &s->cdef[i];
        nmol += (unsigned long)cnt[i];
        double bal[3] = {0, 0, 0};
        for (int k = 0; k < ci->nch; ++k)
            for (int d = 0; d < 3; ++d) bal[d] += ci->ch[k][4] * ci->ch[k][d];
        for (int k = 0; k < ci->ndi; ++k) {
            double ee = 0;
            for (int d = 0; d < 3; ++d) ee += ci->di[k][3 + d] * ci->di[k][3 + d];
            double inv = 1.0 / sqrt(ee);
            for (int d = 0; d < 3; ++d) bal[d] += ci->di[k][6] * ci->di[k][3 + d] * inv;
        }
        double my2 = 0.0;
        for (int d = 0; d < 3; ++d) my2 += bal[d] * bal[d];
        self += my2 * cnt[i];
        for (int j = 0; j < s->ncomp; ++j) {
            const ocomp* cj = &s->cdef[j];
            for (int a = 0; a < ci->nlj; ++a) {
                double t1 = sqrt(ci->lj[a][0] * ci->lj[a][0] + ci->lj[a][1] * ci->lj[a][1] + ci->lj[a][2] * ci->lj[a][2]);
                for (int b = 0; b < cj->nlj; ++b) {
                    double t2 = sqrt(cj->lj[b][0] * cj->lj[b][0] + cj->lj[b][1] * cj->lj[b][1] +
                                     cj->lj[b][2] * cj->lj[b][2]);
                    if (t1 + t2 >= rclj) return MD_ERR_ARG;  /* cut-off too small for the correction */
                    const int g = (ci->ljoff + a) * s->nlj + cj->ljoff + b;
                    if (s->shift6[g] != 0.0) continue;
                    double fac = cnt[i] * cnt[j] * s->eps24[g], s2 = s->sig2[g];
                    if (t1 == 0. && t2 == 0.) {
                        U += fac * (tl_cc_u(-6, rclj, s2) - tl_cc_u(-3, rclj, s2));
                        W += fac * (tl_cc_v(-6, rclj, s2) - tl_cc_v(-3, rclj, s2));
                    } else if (t1 != 0. && t2 != 0.) {
                        U += fac * (tl_ss_u(-6, rclj, s2, t1, t2) - tl_ss_u(-3, rclj, s2, t1, t2));
                        W += fac * (tl_ss_v(-6, rclj, s2, t1, t2) - tl_ss_v(-3, rclj, s2, t1, t2));
                    } else {
                        double t = t2 == 0. ? t1 : t2;
                        U += fac * (tl_cs_u(-6, rclj, s2, t) - tl_cs_u(-3, rclj, s2, t));
                        W += fac * (tl_cs_v(-6, rclj, s2, t) - tl_cs_v(-3, rclj, s2, t));
                    }
                }
            }
        }
    }
    const double vol = (s->cfg.box_max[0] - s->cfg.box_min[0]) * (s->cfg.box_max[1] - s->cfg.box_min[1]) *
                       (s->cfg.box_max[2] - s->cfg.box_min[2]);
    const double rho = (double)nmol / vol;
    const double pi = 3.14159265358979323846;  /* M_PI */
    const double fac = pi * rho / (3. * (double)nmol);
    const double epsRFInvrc3 = 2. * (s->cfg.eps_rf - 1.) / ((rc * rc * rc) * (2. * s->cfg.eps_rf + 1.));
    const double selfterm = -0.5 * epsRFInvrc3 * self;
    *upot_corr = fac * U + selfterm;
    *virial_corr = -fac * W + 3. * selfterm;
    return MD_OK;
}
