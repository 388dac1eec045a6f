/*
 * Test infrastructure: the C-ABI entry points the case façade calls
 * (include/sphdem.h), served by the CPU oracle port instead of the device
 * library.  tests/test_facade.py links a case directory's unmodified hooks
 * against this library, where the reference's case sources exist and no GPU
 * does, to run them end to end through the façade's host mirror; the numbers
 * are the oracle's, so what the test checks is the façade's hook plumbing.
 * Nothing of the product links it.
 */
#include <cstring>
#include <string>

#include "sphdem.h"

extern "C" {
int oracle_create(const SphDemConfig *cfg, const SphDemParticles *init, void **out);
void oracle_destroy(void *h);
int oracle_phase(void *h, int phase);
int oracle_get(void *h, SphDemParticles *o);
int oracle_set(void *h, uint32_t mask, const SphDemParticles *in);
int oracle_globals(void *h, SphDemGlobals *g);
int oracle_set_globals(void *h, const SphDemGlobals *g);
int oracle_pairs(void *h, int kind, int64_t *offs, int32_t *idx, int64_t cap, int64_t *npairs);
int oracle_insert(void *h, const SphDemParticles *in, int64_t *out_idx);
int oracle_mark_for_deletion(void *h, const int64_t *idx, int64_t k);
int oracle_output_vars(void *h, SphDemOutputVars *o);
int oracle_rebuild(void *h);
const char *oracle_last_error(void);
}

struct sphdem_ctx {
    void *o = nullptr;
    std::string err;
};

namespace {
int fail(sphdem_handle h, int rc) {
    if (h) h->err = oracle_last_error();
    return rc;
}
}  // namespace

extern "C" {

int sphdem_create(const SphDemConfig *cfg, const SphDemParticles *init, int64_t, sphdem_handle *out) {
    sphdem_handle h = new sphdem_ctx;
    const int rc = oracle_create(cfg, init, &h->o);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return SPHDEM_OK;
}

int sphdem_destroy(sphdem_handle h) {
    if (h) oracle_destroy(h->o);
    delete h;
    return SPHDEM_OK;
}

int sphdem_phase(sphdem_handle h, int phase) {
    const int rc = oracle_phase(h->o, phase);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

/* only the fields the mask selects, as the device library does */
int sphdem_get_fields(sphdem_handle h, uint32_t mask, SphDemParticles *out) {
    SphDemParticles o = *out;
    if (!(mask & SPHDEM_FIELD_IAM)) o.iam = nullptr;
    if (!(mask & SPHDEM_FIELD_R)) o.r = nullptr;
    if (!(mask & SPHDEM_FIELD_V)) o.v = nullptr;
    if (!(mask & SPHDEM_FIELD_VHAT)) o.vhat = nullptr;
    if (!(mask & SPHDEM_FIELD_MASS)) o.mass = nullptr;
    if (!(mask & SPHDEM_FIELD_DENS)) o.dens = nullptr;
    if (!(mask & SPHDEM_FIELD_H)) o.h = nullptr;
    if (!(mask & SPHDEM_FIELD_F)) o.f = o.fp = o.fv = o.fb = nullptr;
    if (!(mask & SPHDEM_FIELD_DDDT)) o.dddt = nullptr;
    if (!(mask & SPHDEM_FIELD_PRESS)) o.press = o.pdr2 = nullptr;
    if (!(mask & SPHDEM_FIELD_COUPLING))
        o.porosity = o.dporositydt = o.shep_sum = o.fdrag = o.fvel = o.grad_porosity = nullptr;
    if (!(mask & SPHDEM_FIELD_OMEGA)) o.omega = nullptr;
    if (!(mask & SPHDEM_FIELD_V0)) o.v0 = o.vhat0 = nullptr;
    if (!(mask & SPHDEM_FIELD_NORMALS)) o.norm1 = o.norm2 = o.norm3 = nullptr;
    if (!(mask & SPHDEM_FIELD_RADIUS)) o.radius = nullptr;
    if (!(mask & SPHDEM_FIELD_ENERGY)) o.u = o.dudt = o.e_visc = o.de_visc_dt = nullptr;
    const int rc = oracle_get(h->o, &o);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

int sphdem_set_fields(sphdem_handle h, uint32_t mask, const SphDemParticles *in) {
    const int rc = oracle_set(h->o, mask, in);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

int sphdem_get_globals(sphdem_handle h, SphDemGlobals *out) { return oracle_globals(h->o, out); }
int sphdem_set_globals(sphdem_handle h, const SphDemGlobals *in) { return oracle_set_globals(h->o, in); }

int sphdem_pairs(sphdem_handle h, int kind, int64_t *offsets, int32_t *idx, int64_t cap, int64_t *n_pairs) {
    const int rc = oracle_pairs(h->o, kind, offsets, idx, cap, n_pairs);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

int sphdem_insert_particles(sphdem_handle h, const SphDemParticles *in, int64_t *out_idx) {
    const int rc = oracle_insert(h->o, in, out_idx);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

int sphdem_mark_for_deletion(sphdem_handle h, const int64_t *idx, int64_t k) {
    const int rc = oracle_mark_for_deletion(h->o, idx, k);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

int sphdem_rebuild(sphdem_handle h) {
    const int rc = oracle_rebuild(h->o);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

int sphdem_output_vars(sphdem_handle h, SphDemOutputVars *out) {
    const int rc = oracle_output_vars(h->o, out);
    return rc ? fail(h, rc) : SPHDEM_OK;
}

int sphdem_last_error(sphdem_handle h, char *buf, size_t len) {
    if (!buf || !len) return SPHDEM_ERR_INVALID;
    const std::string &e = h ? h->err : std::string();
    std::strncpy(buf, e.c_str(), len - 1);
    buf[len - 1] = 0;
    return SPHDEM_OK;
}

}  // extern "C"
