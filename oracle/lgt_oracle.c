/*
 * lgt_oracle.c -- CPU restatement of the exact-diagonalisation (ED) path of
 * NoaFeldman/LGT: basis enumeration, packed keys, the sparse Hamiltonian of
 * finite_ed.jl and of the plaquette + Jordan-Wigner term list, and the
 * measure_ED observables.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA library is checked
 * against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it, and only as the checker or as the timed CPU baseline; the
 * product (lgt_gb300/) never links or calls it.
 *
 * Parity status.  Julia is not installed where this was written, so the
 * reference cannot be run.  The integer layer restated here follows
 * finite_ed.jl:80-322 step by step (same loops, same visiting order, same
 * dictionary semantics), and is pinned by (i) the sector dimensions and
 * nonzero counts of the reference's staggered sectors, and (ii) an
 * independent full-tensor-product construction of the same Hamiltonian from
 * the reference's local operators (u1_lgt_hamiltonian.jl:111-163,605-618,
 * mps_lgt.jl:83-116, matter_gauge_entanglement_pjw.jl:82-147) projected onto
 * this basis (tests/test_oracle_fullspace.py).  Krylov results (eigsolve /
 * exponentiate of KrylovKit 0.10.2) are "parity unpinned": no reference test
 * stores them.
 *
 * Array conventions follow Julia's column-major storage:
 *   n_f[ix,iy] -> nf[(ix-1) + (iy-1)*nx]          (nx x ny)
 *   e_R[ix,iy] -> eR[(ix-1) + (iy-1)*(nx-1)]      ((nx-1) x ny)
 *   e_U[ix,iy] -> eU[(ix-1) + (iy-1)*nx]          (nx x (ny-1))
 * All indices returned by this file are 0-based (reference index - 1).
 *
 * Build: gcc -O2 -ffp-contract=off -shared -fPIC (see oracle/build.py).
 * -ffp-contract=off keeps every multiply and add separately rounded, as
 * Julia does, so the diagonal sums below are bit-identical to the reference.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAX_SITES 32
#define ORC_MAX_LINKS 64

enum { ORC_MODEL_REF = 0, ORC_MODEL_PJW = 1 };

/* ------------------------------------------------------------------------- */
/* Small open-addressing hash map int64 key -> int64 value (the Dict of     */
/* finite_ed.jl:132).                                                         */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint64_t* keys;
    int64_t* vals;
    uint8_t* used;
    int64_t cap;
    int64_t n;
} orc_map;

static uint64_t orc_hash(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

static int orc_map_init(orc_map* m, int64_t cap) {
    m->cap = cap;
    m->n = 0;
    m->keys = (uint64_t*)calloc((size_t)cap, sizeof(uint64_t));
    m->vals = (int64_t*)calloc((size_t)cap, sizeof(int64_t));
    m->used = (uint8_t*)calloc((size_t)cap, 1);
    return (m->keys && m->vals && m->used) ? 0 : -1;
}

static void orc_map_free(orc_map* m) {
    free(m->keys);
    free(m->vals);
    free(m->used);
    memset(m, 0, sizeof(*m));
}

static int64_t orc_map_get(const orc_map* m, uint64_t k) {
    uint64_t h = orc_hash(k) & (uint64_t)(m->cap - 1);
    while (m->used[h]) {
        if (m->keys[h] == k) return m->vals[h];
        h = (h + 1) & (uint64_t)(m->cap - 1);
    }
    return -1;
}

static int orc_map_put(orc_map* m, uint64_t k, int64_t v);

static int orc_map_grow(orc_map* m) {
    orc_map n2;
    if (orc_map_init(&n2, m->cap * 2)) return -1;
    for (int64_t i = 0; i < m->cap; i++)
        if (m->used[i]) orc_map_put(&n2, m->keys[i], m->vals[i]);
    orc_map_free(m);
    *m = n2;
    return 0;
}

static int orc_map_put(orc_map* m, uint64_t k, int64_t v) {
    if (2 * (m->n + 1) > m->cap && orc_map_grow(m)) return -1;
    uint64_t h = orc_hash(k) & (uint64_t)(m->cap - 1);
    while (m->used[h]) {
        if (m->keys[h] == k) {
            m->vals[h] = v;
            return 0;
        }
        h = (h + 1) & (uint64_t)(m->cap - 1);
    }
    m->used[h] = 1;
    m->keys[h] = k;
    m->vals[h] = v;
    m->n++;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Geometry helpers                                                          */
/* ------------------------------------------------------------------------- */
#define NF(a, ix, iy) (a)[((ix)-1) + ((iy)-1) * nx]
#define ER(a, ix, iy) (a)[((ix)-1) + ((iy)-1) * (nx - 1)]
#define EU(a, ix, iy) (a)[((ix)-1) + ((iy)-1) * nx]

/* Bits needed for one link digit e+dg in [0, 2dg]. */
int orc_digit_bits(int dg) {
    int w = 1;
    while ((1 << w) < 2 * dg + 1) w++;
    return w;
}

/*
 * _encode, finite_ed.jl:80-97.  n_f bits first (iy outer, ix inner), then
 * 2-bit (e+1) fields for e_R (iy outer, ix = 1..nx-1), then for e_U
 * (iy = 1..ny-1 outer, ix inner).  Int64 in the reference: bit 63 may be set
 * (4x4 lattice), the bit pattern is returned unchanged.
 */
int64_t orc_encode(int nx, int ny, const int8_t* nf, const int8_t* eR, const int8_t* eU) {
    uint64_t key = 0;
    int off = 0;
    for (int iy = 1; iy <= ny; iy++)
        for (int ix = 1; ix <= nx; ix++) {
            key |= (uint64_t)(int64_t)NF(nf, ix, iy) << off;
            off += 1;
        }
    for (int iy = 1; iy <= ny; iy++)
        for (int ix = 1; ix <= nx - 1; ix++) {
            key |= (uint64_t)(int64_t)(ER(eR, ix, iy) + 1) << off;
            off += 2;
        }
    for (int iy = 1; iy <= ny - 1; iy++)
        for (int ix = 1; ix <= nx; ix++) {
            key |= (uint64_t)(int64_t)(EU(eU, ix, iy) + 1) << off;
            off += 2;
        }
    return (int64_t)key;
}

/*
 * Order key: (fermion mask << w*N_U) | e_U digits (e+dg), iy outer, ix
 * inner, the first link most significant.  The reference indexes states in
 * discovery order (finite_ed.jl:138,174-200,227-231): masks ascending, then
 * e_U rows lexicographic with each value ascending from -dg.  This key is
 * strictly increasing in that order, so "rank in the sorted key list" equals
 * "reference index - 1".  (The _encode key above is not monotone in it.)
 */
uint64_t orc_order_key(int nx, int ny, int dg, const int8_t* nf, const int8_t* eU) {
    int w = orc_digit_bits(dg);
    uint64_t mask = 0, dig = 0;
    for (int iy = 1; iy <= ny; iy++)
        for (int ix = 1; ix <= nx; ix++)
            mask |= (uint64_t)NF(nf, ix, iy) << ((iy - 1) * nx + (ix - 1));
    for (int iy = 1; iy <= ny - 1; iy++)
        for (int ix = 1; ix <= nx; ix++) dig = (dig << w) | (uint64_t)(EU(eU, ix, iy) + dg);
    int nU = nx * (ny - 1);
    return (nU * w >= 64) ? dig : ((mask << (nU * w)) | dig); /* callers keep ns + w*nU <= 64 */
}

/* ------------------------------------------------------------------------- */
/* Basis: build_basis, finite_ed.jl:125-232                                  */
/* ------------------------------------------------------------------------- */
typedef struct {
    int nx, ny, dg;
    int64_t n, cap;
    uint64_t* okeys;
    int64_t* rkeys;
    int8_t *nf, *eR, *eU; /* n x (nx*ny), n x ((nx-1)*ny), n x (nx*(ny-1)) */
    orc_map dict;         /* key_dict: _encode key (dg==1) or order key -> index */
    /* scratch for the recursion */
    int8_t cnf[ORC_MAX_SITES], ceR[ORC_MAX_SITES], ceU[ORC_MAX_SITES];
    int q[ORC_MAX_SITES];
    int S[ORC_MAX_SITES];
    int err;
} orc_basis;

static uint64_t orc_dict_key(const orc_basis* b, const int8_t* nf, const int8_t* eR, const int8_t* eU) {
    /* The reference keys its Dict by _encode.  That key is only injective for
       dg == 1 (2-bit fields); for dg > 1 the oracle keys by the order key,
       which is what the GPU library defines for dg > 1. */
    if (b->dg == 1) return (uint64_t)orc_encode(b->nx, b->ny, nf, eR, eU);
    return orc_order_key(b->nx, b->ny, b->dg, nf, eU);
}

static int orc_push_state(orc_basis* b) {
    int nx = b->nx, ny = b->ny;
    int ns = nx * ny, nr = (nx - 1) * ny, nu = nx * (ny - 1);
    uint64_t k = orc_dict_key(b, b->cnf, b->ceR, b->ceU);
    if (orc_map_get(&b->dict, k) >= 0) return 0; /* haskey: skip (finite_ed.jl:228) */
    if (b->n == b->cap) {
        int64_t nc = b->cap ? 2 * b->cap : 1024;
        uint64_t* ok = (uint64_t*)realloc(b->okeys, (size_t)nc * sizeof(uint64_t));
        if (ok) b->okeys = ok;
        int64_t* rk = (int64_t*)realloc(b->rkeys, (size_t)nc * sizeof(int64_t));
        if (rk) b->rkeys = rk;
        int8_t* a = (int8_t*)realloc(b->nf, (size_t)nc * (ns ? ns : 1));
        if (a) b->nf = a;
        int8_t* r = (int8_t*)realloc(b->eR, (size_t)nc * (nr ? nr : 1));
        if (r) b->eR = r;
        int8_t* u = (int8_t*)realloc(b->eU, (size_t)nc * (nu ? nu : 1));
        if (u) b->eU = u;
        if (!ok || !rk || !a || !r || !u) return -1;
        b->cap = nc;
    }
    int64_t i = b->n;
    memcpy(b->nf + i * ns, b->cnf, (size_t)ns);
    if (nr) memcpy(b->eR + i * nr, b->ceR, (size_t)nr);
    if (nu) memcpy(b->eU + i * nu, b->ceU, (size_t)nu);
    b->okeys[i] = orc_order_key(nx, ny, b->dg, b->cnf, b->ceU);
    b->rkeys[i] = (b->dg == 1) ? orc_encode(nx, ny, b->cnf, b->ceR, b->ceU) : 0;
    if (orc_map_put(&b->dict, k, i)) return -1;
    b->n++;
    return 0;
}

/* _derive_and_check_eR!, finite_ed.jl:202-232 */
static void orc_derive_and_check(orc_basis* b) {
    int nx = b->nx, ny = b->ny, dg = b->dg;
    for (int iy = 1; iy <= ny; iy++) {
        int acc = 0;
        for (int ix = 1; ix <= nx; ix++) {
            int eu_now = (iy < ny) ? EU(b->ceU, ix, iy) : 0;
            int eu_prev = (iy > 1) ? EU(b->ceU, ix, iy - 1) : 0;
            int d = b->q[(ix - 1) + (iy - 1) * nx] - eu_now + eu_prev;
            acc += d;
            if (ix < nx) {
                if (-dg <= acc && acc <= dg)
                    ER(b->ceR, ix, iy) = (int8_t)acc;
                else
                    return;
            } else if (acc != 0) {
                return;
            }
        }
    }
    if (orc_push_state(b)) b->err = 1;
}

static void orc_eU_row(orc_basis* b, int iy);

/* _eU_inner!, finite_ed.jl:183-200 */
static void orc_eU_inner(orc_basis* b, int iy, int ix, int partial) {
    int nx = b->nx, dg = b->dg;
    if (ix == nx) {
        int last = b->S[iy - 1] - partial;
        if (-dg <= last && last <= dg) {
            EU(b->ceU, nx, iy) = (int8_t)last;
            orc_eU_row(b, iy + 1);
        }
        return;
    }
    for (int v = -dg; v <= dg; v++) {
        EU(b->ceU, ix, iy) = (int8_t)v;
        orc_eU_inner(b, iy, ix + 1, partial + v);
    }
}

/* _eU_row!, finite_ed.jl:172-181 */
static void orc_eU_row(orc_basis* b, int iy) {
    if (b->err) return;
    if (iy == b->ny) {
        orc_derive_and_check(b);
        return;
    }
    orc_eU_inner(b, iy, 1, 0);
}

/*
 * build_basis, finite_ed.jl:125-162.  g_charges is nx x ny column-major.
 * Returns NULL on an inconsistent sector (the reference's @assert at :127)
 * or on a lattice beyond this oracle's limits.
 */
void* orc_basis_new(int nx, int ny, int dg, const int32_t* g_charges) {
    if (nx < 1 || ny < 1 || dg < 1 || nx * ny > 30 || (nx - 1) * ny > ORC_MAX_SITES ||
        nx * (ny - 1) > ORC_MAX_SITES)
        return NULL;
    int ns = nx * ny;
    if (ns + orc_digit_bits(dg) * nx * (ny - 1) > 64) return NULL; /* order key width */
    long gsum = 0;
    for (int i = 0; i < ns; i++) gsum += g_charges[i];
    long nft = -gsum;
    if (nft < 0 || nft > ns) return NULL;
    orc_basis* b = (orc_basis*)calloc(1, sizeof(orc_basis));
    if (!b) return NULL;
    b->nx = nx;
    b->ny = ny;
    b->dg = dg;
    if (orc_map_init(&b->dict, 1024)) {
        free(b);
        return NULL;
    }
    for (uint64_t mask = 0; mask < (1ULL << ns); mask++) {
        if (__builtin_popcountll(mask) != nft) continue;
        for (int iy = 1; iy <= ny; iy++)
            for (int ix = 1; ix <= nx; ix++)
                NF(b->cnf, ix, iy) = (int8_t)((mask >> ((iy - 1) * nx + (ix - 1))) & 1);
        for (int i = 0; i < ns; i++) b->q[i] = b->cnf[i] + g_charges[i];
        int s = 0;
        for (int iy = 1; iy <= ny; iy++) {
            int r = 0;
            for (int ix = 1; ix <= nx; ix++) r += b->q[(ix - 1) + (iy - 1) * nx];
            s += r;
            b->S[iy - 1] = s;
        }
        if (b->S[ny - 1] != 0) continue;
        orc_eU_row(b, 1);
        if (b->err) break;
    }
    if (b->err) {
        orc_map_free(&b->dict);
        free(b->okeys);
        free(b->rkeys);
        free(b->nf);
        free(b->eR);
        free(b->eU);
        free(b);
        return NULL;
    }
    return b;
}

int64_t orc_basis_dim(const void* h) { return ((const orc_basis*)h)->n; }

void orc_basis_copy(const void* h, uint64_t* okeys, int64_t* rkeys, int8_t* nf, int8_t* eR, int8_t* eU) {
    const orc_basis* b = (const orc_basis*)h;
    int ns = b->nx * b->ny, nr = (b->nx - 1) * b->ny, nu = b->nx * (b->ny - 1);
    if (okeys) memcpy(okeys, b->okeys, (size_t)b->n * sizeof(uint64_t));
    if (rkeys) memcpy(rkeys, b->rkeys, (size_t)b->n * sizeof(int64_t));
    if (nf) memcpy(nf, b->nf, (size_t)(b->n * ns));
    if (eR && nr) memcpy(eR, b->eR, (size_t)(b->n * nr));
    if (eU && nu) memcpy(eU, b->eU, (size_t)(b->n * nu));
}

/* key_dict lookup of an encoded key (dg == 1) or order key; -1 when absent. */
int64_t orc_basis_lookup(const void* h, uint64_t key) { return orc_map_get(&((const orc_basis*)h)->dict, key); }

void orc_basis_free(void* h) {
    orc_basis* b = (orc_basis*)h;
    if (!b) return;
    orc_map_free(&b->dict);
    free(b->okeys);
    free(b->rkeys);
    free(b->nf);
    free(b->eR);
    free(b->eU);
    free(b);
}

/* ------------------------------------------------------------------------- */
/* Hamiltonian: build_hamiltonian, finite_ed.jl:252-322 (model REF), and the */
/* plaquette + Jordan-Wigner term list lgt_terms_plaqjw_cs,                  */
/* matter_gauge_entanglement_pjw.jl:82-147 (model PJW).                      */
/* ------------------------------------------------------------------------- */

/*
 * Column snake, decoupling_U_soe.jl:41-54: column ix outer, iy ascending for
 * odd ix and descending for even ix.  1-based position of (ix,iy).
 */
static int orc_snake_pos(int nx, int ny, int ix, int iy) {
    (void)nx;
    return (ix - 1) * ny + ((ix & 1) ? iy : (ny + 1 - iy));
}

/* Parity (-1)^(sum n_f) over sites strictly between two snake positions. */
static int orc_jw_sign(int nx, int ny, const int8_t* nf, int ax, int ay, int bx, int by) {
    int pa = orc_snake_pos(nx, ny, ax, ay), pb = orc_snake_pos(nx, ny, bx, by);
    int lo = pa < pb ? pa : pb, hi = pa < pb ? pb : pa;
    int par = 0;
    for (int iy = 1; iy <= ny; iy++)
        for (int ix = 1; ix <= nx; ix++) {
            int p = orc_snake_pos(nx, ny, ix, iy);
            if (p > lo && p < hi) par ^= NF(nf, ix, iy);
        }
    return par ? -1 : 1;
}

typedef struct {
    int64_t n, cap;
    int64_t *I, *J;
    double* V;
    int err;
} orc_coo;

static void orc_coo_push(orc_coo* c, int64_t i, int64_t j, double v) {
    if (c->err) return;
    if (c->n == c->cap) {
        int64_t nc = c->cap ? 2 * c->cap : 4096;
        int64_t* I2 = (int64_t*)realloc(c->I, (size_t)nc * sizeof(int64_t));
        if (I2) c->I = I2;
        int64_t* J2 = (int64_t*)realloc(c->J, (size_t)nc * sizeof(int64_t));
        if (J2) c->J = J2;
        double* V2 = (double*)realloc(c->V, (size_t)nc * sizeof(double));
        if (V2) c->V = V2;
        if (!I2 || !J2 || !V2) {
            c->err = 1;
            return;
        }
        c->cap = nc;
    }
    c->I[c->n] = i;
    c->J[c->n] = j;
    c->V[c->n] = v;
    c->n++;
}

/*
 * The body of the reference's loop over states (finite_ed.jl:262-319) for
 * one state idx: its diagonal, its forward hops and (model PJW) its
 * plaquette moves, each move pushing (jdx, idx) and (idx, jdx) as the
 * reference does.  With only_row >= 0, only the triplets of that row are
 * kept (the row-restricted build below).  Returns 0, or 1 when a moved
 * state is missing from the basis (which the Gauss law rules out).
 */
static int orc_ham_state(const orc_basis* b, int model, double g, double t, double m,
                         int64_t idx, int64_t only_row, orc_coo* c) {
    int nx = b->nx, ny = b->ny, dg = b->dg;
    int ns = nx * ny, nr = (nx - 1) * ny, nu = nx * (ny - 1);
    int8_t wnf[ORC_MAX_SITES], weR[ORC_MAX_SITES], weU[ORC_MAX_SITES];
    const double invg2 = 1.0 / (2.0 * (g * g)); /* matter_gauge_entanglement_pjw.jl:131 */
    const int8_t* snf = b->nf + idx * ns;
    const int8_t* seR = b->eR + idx * nr;
    const int8_t* seU = b->eU + idx * nu;
#define ORC_PUSH(i, j, v) \
    do { if (only_row < 0 || (i) == only_row) orc_coo_push(c, (i), (j), (v)); } while (0)
    /* Diagonal, finite_ed.jl:265-276: same loop, same rounding order. */
    double E = 0.0;
    for (int iy = 1; iy <= ny; iy++)
        for (int ix = 1; ix <= nx; ix++) {
            if (ix < nx) {
                double e = (double)ER(seR, ix, iy);
                E += ((g * g) / 2) * (e * e);
            }
            if (iy < ny) {
                double e = (double)EU(seU, ix, iy);
                E += ((g * g) / 2) * (e * e);
            }
            int stag = ((ix + iy) % 2 == 0) ? 1 : -1;
            E += (m * stag) * (double)NF(snf, ix, iy);
        }
    ORC_PUSH(idx, idx, E);
    /* Horizontal forward hops, finite_ed.jl:279-297 */
    for (int iy = 1; iy <= ny; iy++)
        for (int ix = 1; ix <= nx - 1; ix++) {
            int e = ER(seR, ix, iy);
            int nL = NF(snf, ix, iy), nR = NF(snf, ix + 1, iy);
            if (nL == 0 && nR == 1 && e < dg) {
                memcpy(wnf, snf, (size_t)ns);
                memcpy(weR, seR, (size_t)nr);
                if (nu) memcpy(weU, seU, (size_t)nu);
                NF(wnf, ix, iy) = 1;
                NF(wnf, ix + 1, iy) = 0;
                ER(weR, ix, iy) = (int8_t)(e + 1);
                int64_t jdx = orc_map_get(&b->dict, orc_dict_key(b, wnf, weR, weU));
                if (jdx < 0) return 1;
                double v = -t;
                if (model == ORC_MODEL_PJW) v = -t * orc_jw_sign(nx, ny, snf, ix, iy, ix + 1, iy);
                ORC_PUSH(jdx, idx, v);
                ORC_PUSH(idx, jdx, v);
            }
        }
    /* Vertical forward hops, finite_ed.jl:300-318 (chain-adjacent on the
       column snake, so no Jordan-Wigner string in the PJW model) */
    for (int iy = 1; iy <= ny - 1; iy++)
        for (int ix = 1; ix <= nx; ix++) {
            int e = EU(seU, ix, iy);
            int nD = NF(snf, ix, iy), nU = NF(snf, ix, iy + 1);
            if (nD == 0 && nU == 1 && e < dg) {
                memcpy(wnf, snf, (size_t)ns);
                if (nr) memcpy(weR, seR, (size_t)nr);
                memcpy(weU, seU, (size_t)nu);
                NF(wnf, ix, iy) = 1;
                NF(wnf, ix, iy + 1) = 0;
                EU(weU, ix, iy) = (int8_t)(e + 1);
                int64_t jdx = orc_map_get(&b->dict, orc_dict_key(b, wnf, weR, weU));
                if (jdx < 0) return 1;
                double v = -t;
                if (model == ORC_MODEL_PJW) v = -t * orc_jw_sign(nx, ny, snf, ix, iy, ix, iy + 1);
                ORC_PUSH(jdx, idx, v);
                ORC_PUSH(idx, jdx, v);
            }
        }
    /* Magnetic plaquette, matter_gauge_entanglement_pjw.jl:130-144:
       -(1/2g^2)(W + W^dagger), W = U^dag on e_R(ix,iy) (bottom), U on
       e_U(ix,iy) (left), U^dag on e_U(ix+1,iy) (right), U on e_R(ix,iy+1)
       (top).  U|e> = |e+1>, zero at e = dg (u1_lgt_hamiltonian.jl:124-131).
       W maps state idx to jdx; W^dagger maps jdx back, giving the mirrored
       entry. */
    if (model == ORC_MODEL_PJW) {
        for (int iy = 1; iy <= ny - 1; iy++)
            for (int ix = 1; ix <= nx - 1; ix++) {
                int eb = ER(seR, ix, iy), et = ER(seR, ix, iy + 1);
                int el = EU(seU, ix, iy), er = EU(seU, ix + 1, iy);
                if (eb - 1 < -dg || el + 1 > dg || er - 1 < -dg || et + 1 > dg) continue;
                memcpy(wnf, snf, (size_t)ns);
                memcpy(weR, seR, (size_t)nr);
                memcpy(weU, seU, (size_t)nu);
                ER(weR, ix, iy) = (int8_t)(eb - 1);
                EU(weU, ix, iy) = (int8_t)(el + 1);
                EU(weU, ix + 1, iy) = (int8_t)(er - 1);
                ER(weR, ix, iy + 1) = (int8_t)(et + 1);
                int64_t jdx = orc_map_get(&b->dict, orc_dict_key(b, wnf, weR, weU));
                if (jdx < 0) return 1;
                ORC_PUSH(jdx, idx, -invg2);
                ORC_PUSH(idx, jdx, -invg2);
            }
    }
#undef ORC_PUSH
    return 0;
}

static void* orc_coo_done(orc_coo* c) {
    if (c->err) {
        free(c->I);
        free(c->J);
        free(c->V);
        free(c);
        return NULL;
    }
    return c;
}

/*
 * Builds the COO triplets in the reference's push order (0-based).  The
 * caller turns them into CSR/CSC, summing duplicates like SparseArrays'
 * sparse(Is, Js, Vs, N, N) (finite_ed.jl:321); this Hamiltonian has none.
 * Returns NULL on allocation failure or when a hopped state is missing
 * from the basis (which the Gauss law rules out).
 */
void* orc_ham_new(const void* hb, int model, double g, double t, double m) {
    const orc_basis* b = (const orc_basis*)hb;
    orc_coo* c = (orc_coo*)calloc(1, sizeof(orc_coo));
    if (!c) return NULL;
    for (int64_t idx = 0; idx < b->n && !c->err; idx++)
        if (orc_ham_state(b, model, g, t, m, idx, -1, c)) c->err = 1;
    return orc_coo_done(c);
}

/*
 * The triplets of the given rows only, without building the whole matrix
 * (for sampled-row checks of sectors whose full matrix is too large to
 * build in a test).  Row r receives triplets from the loop body of state r
 * itself and of every state whose forward move lands on r; those are found
 * by undoing each possible move of r and looking the result up in the
 * dictionary, then the unchanged loop body (orc_ham_state) runs for each of
 * them, keeping row r's triplets only.  Within a row the triplets come in
 * the order of the sources visited (r first, then the undone moves), not
 * in the full build's order; callers sum duplicates as sparse() would.
 * Agreement with orc_ham_new row by row is checked in the CPU tests.
 */
void* orc_ham_rows(const void* hb, int model, double g, double t, double m, const int64_t* rows,
                   int64_t nrows) {
    const orc_basis* b = (const orc_basis*)hb;
    int nx = b->nx, ny = b->ny, dg = b->dg;
    int ns = nx * ny, nr = (nx - 1) * ny, nu = nx * (ny - 1);
    orc_coo* c = (orc_coo*)calloc(1, sizeof(orc_coo));
    if (!c) return NULL;
    int8_t wnf[ORC_MAX_SITES], weR[ORC_MAX_SITES], weU[ORC_MAX_SITES];
    for (int64_t q = 0; q < nrows && !c->err; q++) {
        const int64_t r = rows[q];
        if (r < 0 || r >= b->n) {
            c->err = 1;
            break;
        }
        if (orc_ham_state(b, model, g, t, m, r, r, c)) {
            c->err = 1;
            break;
        }
        const int8_t* snf = b->nf + r * ns;
        const int8_t* seR = b->eR + r * nr;
        const int8_t* seU = b->eU + r * nu;
#define ORC_SOURCE()                                                                   \
    do {                                                                               \
        int64_t src = orc_map_get(&b->dict, orc_dict_key(b, wnf, weR, weU));           \
        if (src >= 0 && orc_ham_state(b, model, g, t, m, src, r, c)) c->err = 1;       \
    } while (0)
        /* undone horizontal hops: r has the fermion on L, none on R, e > -dg */
        for (int iy = 1; iy <= ny; iy++)
            for (int ix = 1; ix <= nx - 1; ix++) {
                int e = ER(seR, ix, iy);
                if (NF(snf, ix, iy) == 1 && NF(snf, ix + 1, iy) == 0 && e > -dg) {
                    memcpy(wnf, snf, (size_t)ns);
                    memcpy(weR, seR, (size_t)nr);
                    if (nu) memcpy(weU, seU, (size_t)nu);
                    NF(wnf, ix, iy) = 0;
                    NF(wnf, ix + 1, iy) = 1;
                    ER(weR, ix, iy) = (int8_t)(e - 1);
                    ORC_SOURCE();
                }
            }
        /* undone vertical hops */
        for (int iy = 1; iy <= ny - 1; iy++)
            for (int ix = 1; ix <= nx; ix++) {
                int e = EU(seU, ix, iy);
                if (NF(snf, ix, iy) == 1 && NF(snf, ix, iy + 1) == 0 && e > -dg) {
                    memcpy(wnf, snf, (size_t)ns);
                    if (nr) memcpy(weR, seR, (size_t)nr);
                    memcpy(weU, seU, (size_t)nu);
                    NF(wnf, ix, iy) = 0;
                    NF(wnf, ix, iy + 1) = 1;
                    EU(weU, ix, iy) = (int8_t)(e - 1);
                    ORC_SOURCE();
                }
            }
        /* undone plaquette moves W (model PJW) */
        if (model == ORC_MODEL_PJW) {
            for (int iy = 1; iy <= ny - 1; iy++)
                for (int ix = 1; ix <= nx - 1; ix++) {
                    int eb = ER(seR, ix, iy), et = ER(seR, ix, iy + 1);
                    int el = EU(seU, ix, iy), er = EU(seU, ix + 1, iy);
                    if (eb + 1 > dg || el - 1 < -dg || er + 1 > dg || et - 1 < -dg) continue;
                    memcpy(wnf, snf, (size_t)ns);
                    memcpy(weR, seR, (size_t)nr);
                    memcpy(weU, seU, (size_t)nu);
                    ER(weR, ix, iy) = (int8_t)(eb + 1);
                    EU(weU, ix, iy) = (int8_t)(el - 1);
                    EU(weU, ix + 1, iy) = (int8_t)(er + 1);
                    ER(weR, ix, iy + 1) = (int8_t)(et - 1);
                    ORC_SOURCE();
                }
        }
#undef ORC_SOURCE
    }
    return orc_coo_done(c);
}

int64_t orc_ham_ntriplets(const void* h) { return ((const orc_coo*)h)->n; }

void orc_ham_copy(const void* h, int64_t* I, int64_t* J, double* V) {
    const orc_coo* c = (const orc_coo*)h;
    memcpy(I, c->I, (size_t)c->n * sizeof(int64_t));
    memcpy(J, c->J, (size_t)c->n * sizeof(int64_t));
    memcpy(V, c->V, (size_t)c->n * sizeof(double));
}

void orc_ham_free(void* h) {
    orc_coo* c = (orc_coo*)h;
    if (!c) return;
    free(c->I);
    free(c->J);
    free(c->V);
    free(c);
}

/* ------------------------------------------------------------------------- */
/* Observables                                                               */
/* ------------------------------------------------------------------------- */

/*
 * measure_ED, finite_ed.jl:369-393: site grids of <n_f> and <E^2> from the
 * probabilities p = |psi|^2 (nf_grid, E2_grid are nx x ny column-major and
 * are overwritten).
 */
void orc_measure(const void* hb, const double* prob, double* nf_grid, double* E2_grid) {
    const orc_basis* b = (const orc_basis*)hb;
    int nx = b->nx, ny = b->ny;
    int ns = nx * ny, nr = (nx - 1) * ny, nu = nx * (ny - 1);
    for (int i = 0; i < ns; i++) nf_grid[i] = E2_grid[i] = 0.0;
    for (int64_t idx = 0; idx < b->n; idx++) {
        double p = prob[idx];
        const int8_t* snf = b->nf + idx * ns;
        const int8_t* seR = b->eR + idx * nr;
        const int8_t* seU = b->eU + idx * nu;
        for (int iy = 1; iy <= ny; iy++)
            for (int ix = 1; ix <= nx; ix++) {
                NF(nf_grid, ix, iy) += p * (double)NF(snf, ix, iy);
                double e2 = 0.0;
                if (ix < nx) {
                    double e = (double)ER(seR, ix, iy);
                    e2 += e * e;
                }
                if (iy < ny) {
                    double e = (double)EU(seU, ix, iy);
                    e2 += e * e;
                }
                NF(E2_grid, ix, iy) += p * e2;
            }
    }
}

/*
 * Plaquette expectation per plaquette, <W_p + W_p^dagger> with W_p as in the
 * PJW plaquette term above.  plaq is (nx-1) x (ny-1) column-major.  psi is
 * given as separate real and imaginary parts (im may be NULL).
 * <W + W^dag> = 2 Re sum_i conj(psi[W i]) psi[i].
 */
void orc_plaquette(const void* hb, const double* re, const double* im, double* plaq) {
    const orc_basis* b = (const orc_basis*)hb;
    int nx = b->nx, ny = b->ny, dg = b->dg;
    int ns = nx * ny, nr = (nx - 1) * ny, nu = nx * (ny - 1);
    int8_t weR[ORC_MAX_SITES], weU[ORC_MAX_SITES];
    for (int i = 0; i < (nx - 1) * (ny - 1); i++) plaq[i] = 0.0;
    for (int64_t idx = 0; idx < b->n; idx++) {
        const int8_t* snf = b->nf + idx * ns;
        const int8_t* seR = b->eR + idx * nr;
        const int8_t* seU = b->eU + idx * nu;
        for (int iy = 1; iy <= ny - 1; iy++)
            for (int ix = 1; ix <= nx - 1; ix++) {
                int eb = ER(seR, ix, iy), et = ER(seR, ix, iy + 1);
                int el = EU(seU, ix, iy), er = EU(seU, ix + 1, iy);
                if (eb - 1 < -dg || el + 1 > dg || er - 1 < -dg || et + 1 > dg) continue;
                memcpy(weR, seR, (size_t)nr);
                memcpy(weU, seU, (size_t)nu);
                ER(weR, ix, iy) = (int8_t)(eb - 1);
                EU(weU, ix, iy) = (int8_t)(el + 1);
                EU(weU, ix + 1, iy) = (int8_t)(er - 1);
                ER(weR, ix, iy + 1) = (int8_t)(et + 1);
                int64_t j = orc_map_get(&b->dict, orc_dict_key(b, snf, weR, weU));
                if (j < 0) continue;
                double acc = re[j] * re[idx];
                if (im) acc += im[j] * im[idx];
                plaq[(ix - 1) + (iy - 1) * (nx - 1)] += 2.0 * acc;
            }
    }
}
