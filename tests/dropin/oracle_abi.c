/*
 * oracle_abi.c -- TEST INFRASTRUCTURE ONLY.  A stand-in for the engine
 * library (libls1gb300.so) built over the CPU oracle (oracle/md_oracle.c),
 * exporting the part of the C ABI (include/ls1gb300.h) that ls1-MarDyn's
 * drop-in classes call: md_create, md_destroy, md_last_error,
 * md_set_components, md_upload_molecules, md_set_forces,
 * md_download_molecules, md_compute_forces, md_integrate_pre and
 * md_integrate_post.
 *
 * With it the patched MarDyn (<datastructure type="GpuLinkedCells">,
 * <integrator type="GpuLeapfrog">) runs on a host without a GPU, so its glue
 * -- XML selection, the device-context set-up from the ensemble's components
 * and mixing rules, uploads, lazy host-mirror syncs for plugins that iterate,
 * re-uploads after edits, and the Domain sums -- executes and can be compared
 * with the reference's own LinkedCells + Leapfrog run (tests/test_ls1_dropin.py).
 * The product path never uses it.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../../oracle/md_oracle.h"

struct md_ctx {
    md_config cfg;
    orc_sys* s;
};

int md_create(md_ctx** out, const md_config* cfg) {
    if (!out || !cfg) return MD_ERR_ARG;
    md_ctx* c = (md_ctx*)calloc(1, sizeof(md_ctx));
    if (!c) return MD_ERR_ARG;
    c->cfg = *cfg;
    *out = c;
    return MD_OK;
}

int md_destroy(md_ctx* c) {
    if (!c) return MD_ERR_ARG;
    if (c->s) orc_destroy(c->s);
    free(c);
    return MD_OK;
}

const char* md_last_error(const md_ctx* c) {
    (void)c;
    return "oracle stand-in";
}

int md_set_components(md_ctx* c, const md_component* comps, int32_t ncomp, const double* mixing) {
    if (!c || !comps || ncomp < 1) return MD_ERR_ARG;
    if (c->s) orc_destroy(c->s);
    c->s = orc_create(&c->cfg, comps, ncomp, mixing);
    return c->s ? MD_OK : MD_ERR_ARG;
}

int md_upload_molecules(md_ctx* c, int64_t n, const uint64_t* id, const int32_t* comp, const double* r,
                        const double* v, const double* q, const double* L) {
    if (!c || !c->s) return MD_ERR_STATE;
    return orc_set_molecules(c->s, n, id, comp, r, v, q, L);
}

int md_set_forces(md_ctx* c, int64_t n, const double* F, const double* M, const double* Vi) {
    if (!c || !c->s) return MD_ERR_STATE;
    return orc_set_forces(c->s, n, F, M, Vi);
}

/* positions wrapped into the box with the leaving-particle rule, as the engine's download hands them out */
int md_download_molecules(md_ctx* c, int64_t n, uint64_t* id, int32_t* comp, double* r, double* v, double* q,
                          double* L, double* F, double* M, double* Vi) {
    if (!c || !c->s) return MD_ERR_STATE;
    int rc = orc_get_molecules(c->s, n, id, comp, r, v, q, L, F, M, Vi);
    if (rc || !r) return rc;
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            if (!c->cfg.periodic[d]) continue;
            const double lo = c->cfg.box_min[d], hi = c->cfg.box_max[d], len = hi - lo;
            double x = r[3 * i + d];
            if (x < lo) {
                x += len;
                if (x >= hi) x = nextafter(hi, lo);
            } else if (x >= hi) {
                x -= len;
                if (x <= lo) x = lo;
            }
            r[3 * i + d] = x;
        }
    return MD_OK;
}

int md_compute_forces(md_ctx* c, md_forces_out* out) {
    if (!c || !c->s) return MD_ERR_STATE;
    md_bin_stats st;
    double kc[8];
    int rc = orc_rebin_and_halo(c->s, &st);
    if (rc) return rc;
    md_forces_out tmp;
    return orc_forces(c->s, out ? out : &tmp, kc);
}

int md_integrate_pre(md_ctx* c, double dt) {
    if (!c || !c->s) return MD_ERR_STATE;
    return orc_pre(c->s, dt);
}

int md_integrate_post(md_ctx* c, double dt, md_kinetic_out* out) {
    if (!c || !c->s) return MD_ERR_STATE;
    md_kinetic_out tmp;
    return orc_post(c->s, dt, out ? out : &tmp);
}
