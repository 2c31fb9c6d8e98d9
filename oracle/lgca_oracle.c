/*
 * CPU oracle for the lattice-gas hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference algorithm (keva92/lgca).  Every
 * function cites the reference lines it follows.  Used by tests/, by the
 * smoke check and by the benchmark's CPU-baseline leg; never by the product.
 *
 * State format: one byte per cell, bit d = channel d, exactly the reference's
 * Bitset blocks (src/lgca_bitset.h:31-245; bit dir + 8*cell, used at
 * src/omp_lattice.cpp:179,237 and src/lattice.cpp:212).
 */
#include "lgca_oracle.h"
#include "../include/lgca/rng.h"

#include <stdlib.h>
#include <string.h>
#include <math.h>

#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_num_dir(int model)
{
    /* src/lgca_models.h:41 (HPP 4), :234 (FHP-I 6), :441 and :659 (FHP-II/III 7) */
    return model == OR_HPP ? 4 : (model == OR_FHP_I ? 6 : 7);
}

/* Inverse and mirror direction tables: src/lgca_models.h:44-48 (HPP),
 * :239-243 (FHP-I), :446-450 (FHP-II), :664-668 (FHP-III). */
static const int INV_HPP[4] = {2, 3, 0, 1};
static const int MIRX_HPP[4] = {0, 3, 2, 1};
static const int MIRY_HPP[4] = {2, 1, 0, 3};
static const int INV_FHP[7] = {3, 4, 5, 0, 1, 2, 6};
static const int MIRX_FHP[7] = {0, 5, 4, 3, 2, 1, 6};
static const int MIRY_FHP[7] = {3, 2, 1, 0, 5, 4, 6};

static const int *inv_dir(int model) { return model == OR_HPP ? INV_HPP : INV_FHP; }
static const int *mir_x(int model) { return model == OR_HPP ? MIRX_HPP : MIRX_FHP; }
static const int *mir_y(int model) { return model == OR_HPP ? MIRY_HPP : MIRY_FHP; }

#define BIT(v, i) (((v) >> (i)) & 1u)

/* ModelDescriptor<HPP>::collide, src/lgca_models.h:134-152: the two head-on
 * pairs (0,2) and (1,3) swap when exactly one pair is occupied; p unused. */
static uint8_t collide_hpp(uint8_t in)
{
    unsigned n0 = BIT(in, 0), n1 = BIT(in, 1), n2 = BIT(in, 2), n3 = BIT(in, 3);
    unsigned h02 = n0 & n2 & (1u - n1) & (1u - n3); /* 0,2 occupied, 1,3 empty */
    unsigned h13 = n1 & n3 & (1u - n0) & (1u - n2);
    unsigned o0 = n0 - h02 + h13, o1 = n1 - h13 + h02;
    unsigned o2 = n2 - h02 + h13, o3 = n3 - h13 + h02;
    return (uint8_t)(o0 | (o1 << 1) | (o2 << 2) | (o3 << 3) | (in & 0xF0u));
}

/* ModelDescriptor<FHP_I/II/III>::collide, src/lgca_models.h:367-395 (FHP-I),
 * :568-613 (FHP-II) and :786-856 (FHP-III).  Channel letters a..f are
 * channels 1,2,3,4,5,0 and r is the rest channel 6 (:369-375).  The FHP-III
 * terms of :816-839 are evaluated as written; each ANDs a two-body pattern
 * that requires a channel to be empty with a term that requires the same
 * channel to be occupied, so they are identically zero and FHP-III equals
 * FHP-II (checked exhaustively by the tests). */
static uint8_t collide_fhp(int model, uint8_t in, int p_in)
{
    unsigned a = BIT(in, 1), b = BIT(in, 2), c = BIT(in, 3);
    unsigned d = BIT(in, 4), e = BIT(in, 5), f = BIT(in, 0);
    unsigned r = model == OR_FHP_I ? 0u : BIT(in, 6);
    unsigned p = p_in ? 1u : 0u, np = 1u - p;

    /* head-on pairs with every other moving channel empty (:376-378) */
    unsigned db1 = a & d & !(b | c | e | f);
    unsigned db2 = b & e & !(a | c | d | f);
    unsigned db3 = c & f & !(a | b | d | e);
    /* symmetric three-body a,c,e <-> b,d,f (:380) */
    unsigned triple = (a ^ b) & (b ^ c) & (c ^ d) & (d ^ e) & (e ^ f);

    unsigned ra = 0, rb = 0, rc = 0, rd = 0, re = 0, rf = 0;
    unsigned ra2 = 0, rb2 = 0, rc2 = 0, rd2 = 0, re2 = 0, rf2 = 0;
    unsigned spad = 0, spbe = 0, spcf = 0, chad = 0, chbe = 0, chcf = 0;
    if (model != OR_FHP_I) {
        /* rest + one moving -> two moving at +-60 deg (:584-589) */
        ra = r & a & !(b | c | d | e | f);
        rb = r & b & !(a | c | d | e | f);
        rc = r & c & !(a | b | d | e | f);
        rd = r & d & !(a | b | c | e | f);
        re = r & e & !(a | b | c | d | f);
        rf = r & f & !(a | b | c | d | e);
        /* and back (:591-596) */
        ra2 = f & b & !(r | a | c | d | e);
        rb2 = a & c & !(r | b | d | e | f);
        rc2 = b & d & !(r | a | c | e | f);
        rd2 = c & e & !(r | a | b | d | f);
        re2 = d & f & !(r | a | b | c | e);
        rf2 = e & a & !(r | b | c | d | f);
    }
    if (model == OR_FHP_III) {
        /* :816-839, kept literally */
        unsigned adbe = db1 & db2 & !(c | f);
        unsigned adcf = db1 & db3 & !(b | e);
        unsigned becf = db2 & db3 & !(a | d);
        chad = (p & adbe) | (np & adcf) | becf;
        chbe = (p & becf) | (np & adbe) | adcf;
        chcf = (p & adcf) | (np & becf) | adbe;
        unsigned adb = db1 & b & !(c | e | f), adc = db1 & c & !(b | e | f);
        unsigned ade = db1 & e & !(b | c | f), adf = db1 & f & !(b | c | e);
        unsigned bea = db2 & a & !(c | d | f), bec = db2 & c & !(a | d | f);
        unsigned bed = db2 & d & !(a | c | f), bef = db2 & f & !(a | c | d);
        unsigned cfa = db3 & a & !(b | d | e), cfb = db3 & b & !(a | d | e);
        unsigned cfd = db3 & d & !(a | b | e), cfe = db3 & e & !(a | b | d);
        spad = adb | ade | adc | adf | bec | bef | cfb | cfe;
        spbe = bea | bec | bed | bef | adc | adf | cfa | cfd;
        spcf = cfa | cfb | cfd | cfe | adb | ade | bea | bed;
    }

    /* change flags (:382-387, :598-604, :841-847) */
    unsigned cha = triple | db1 | (p & db2) | (np & db3) | ra | rb | rf | ra2 | rb2 | rf2 | spad | chad;
    unsigned chd = triple | db1 | (p & db2) | (np & db3) | rd | rc | re | rd2 | rc2 | re2 | spad | chad;
    unsigned chb = triple | db2 | (p & db3) | (np & db1) | rb | ra | rc | rb2 | ra2 | rc2 | spbe | chbe;
    unsigned che = triple | db2 | (p & db3) | (np & db1) | re | rd | rf | re2 | rd2 | rf2 | spbe | chbe;
    unsigned chc = triple | db3 | (p & db1) | (np & db2) | rc | rb | rd | rc2 | rb2 | rd2 | spcf | chcf;
    unsigned chf = triple | db3 | (p & db1) | (np & db2) | rf | ra | re | rf2 | ra2 | re2 | spcf | chcf;
    unsigned chr = ra | rb | rc | rd | re | rf | ra2 | rb2 | rc2 | rd2 | re2 | rf2;

    unsigned out = (f ^ chf) | ((a ^ cha) << 1) | ((b ^ chb) << 2) | ((c ^ chc) << 3) |
                   ((d ^ chd) << 4) | ((e ^ che) << 5);
    if (model == OR_FHP_I)
        out |= in & 0xC0u; /* channels >= NUM_DIR are never touched */
    else
        out |= ((r ^ chr) << 6) | (in & 0x80u);
    return (uint8_t)out;
}

uint8_t oracle_collide(int model, uint8_t in, int p)
{
    return model == OR_HPP ? collide_hpp(in) : collide_fhp(model, in, p);
}

/* Permute the first D channels: out[d] = in[perm[d]]
 * (bounce_back / bounce_forward_x/y, src/lgca_models.h:184-220, :397-427,
 * :615-645, :858-888). */
static uint8_t permute(int D, const int *perm, uint8_t in)
{
    unsigned out = 0;
    for (int d = 0; d < D; ++d) out |= BIT(in, perm[d]) << d;
    return (uint8_t)(out | (in & (0xFFu << D)));
}

/* Neighbour offset tables of ModelDescriptor<M>(dim_x, dim_y):
 * src/lgca_models.h:79-132 (HPP) and :292-365 / :483-566 / :701-784 (FHP).
 * Index [parity][dir]; the boundary corrections are applied when the pulling
 * cell lies on that edge (src/omp_lattice.cpp:150-176). */
typedef struct {
    long nb[2][7], east[2][7], north[2][7], west[2][7], south[2][7];
} offsets_t;

static void build_offsets(int model, long W, long H, offsets_t *o)
{
    memset(o, 0, sizeof(*o));
    long WH = W * H;
    if (model == OR_HPP) {
        long nb[4] = {1, W, -1, -W};
        for (int par = 0; par < 2; ++par) {
            for (int d = 0; d < 4; ++d) o->nb[par][d] = nb[d];
            o->east[par][2] = W;    /* offset_to_eastern_boundary  */
            o->north[par][3] = WH;  /* offset_to_northern_boundary */
            o->west[par][0] = -W;   /* offset_to_western_boundary  */
            o->south[par][1] = -WH; /* offset_to_southern_boundary */
        }
        return;
    }
    long nbe[6] = {1, W, W - 1, -1, -W - 1, -W};
    long nbo[6] = {1, W + 1, W, -1, -W, -W + 1};
    for (int d = 0; d < 6; ++d) { o->nb[0][d] = nbe[d]; o->nb[1][d] = nbo[d]; }
    /* even rows */
    o->east[0][2] = W; o->east[0][3] = W; o->east[0][4] = W;
    o->north[0][4] = WH; o->north[0][5] = WH;
    o->west[0][0] = -W;
    o->south[0][1] = -WH; o->south[0][2] = -WH + 1;
    /* odd rows */
    o->east[1][3] = W;
    o->north[1][4] = WH; o->north[1][5] = WH;
    o->west[1][0] = -W; o->west[1][1] = -W; o->west[1][5] = -W;
    o->south[1][1] = -WH; o->south[1][2] = -WH;
}

typedef struct { uint8_t coll[2][256], bb[256], bfx[256], bfy[256]; } luts_t;

static void build_luts(int model, luts_t *t)
{
    int D = oracle_num_dir(model);
    for (int s = 0; s < 256; ++s) {
        t->coll[0][s] = oracle_collide(model, (uint8_t)s, 0);
        t->coll[1][s] = oracle_collide(model, (uint8_t)s, 1);
        t->bb[s] = permute(D, inv_dir(model), (uint8_t)s);
        t->bfx[s] = permute(D, mir_x(model), (uint8_t)s);
        t->bfy[s] = permute(D, mir_y(model), (uint8_t)s);
    }
}

static int chirality(const oracle_cfg *cfg, uint64_t key, long x, long y)
{
    if (cfg->chir) return cfg->chir[y * cfg->W + x] != 0;
    uint64_t w = lgca_rng_draw(key, lgca_rng_index((uint32_t)y, (uint32_t)(x >> 6)));
    return (int)((w >> (x & 63)) & 1u);
}

/* OMP_Lattice<M>::collide_and_propagate, src/omp_lattice.cpp:100-249.
 * Pull: channel d of cell comes from cell + offset[INV_DIR[d]] (+ edge
 * corrections).  Update by cell type: FLUID -> collide with the cell's
 * chirality bit (:196-200), SOLID_NO_SLIP -> bounce_back (:204-208),
 * SOLID_SLIP -> unchanged, mirrored in x on the N/S edge rows and then in y
 * on the E/W edge columns, the latter winning at corners (:212-229). */
void oracle_collide_and_propagate(const oracle_cfg *cfg, const int32_t *types,
                                  const uint8_t *state, uint8_t *next, uint64_t t)
{
    const int model = cfg->model, D = oracle_num_dir(model);
    const long W = cfg->W, H = cfg->H, N = W * H;
    const int *inv = inv_dir(model);
    offsets_t o;
    luts_t lut;
    build_offsets(model, W, H, &o);
    build_luts(model, &lut);
    const uint64_t key = lgca_rng_key(cfg->seed, LGCA_STREAM_CHIR, t);

#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long y = 0; y < H; ++y) {
        const int par = (int)(y & 1);
        const int north = y == H - 1, south = y == 0;
        for (long x = 0; x < W; ++x) {
            const long cell = y * W + x;
            const int east = x == W - 1, west = x == 0;
            unsigned in = 0;
            for (int d = 0; d < D; ++d) {
                const int id = inv[d];
                long off = o.nb[par][id];
                if (east) off += o.west[par][id];
                if (north) off += o.south[par][id];
                if (west) off += o.east[par][id];
                if (south) off += o.north[par][id];
                in |= (unsigned)BIT(state[cell + off], d) << d;
            }
            const int ct = types ? types[cell] : OR_FLUID;
            uint8_t out;
            if (ct == OR_FLUID) {
                out = lut.coll[chirality(cfg, key, x, y)][in];
            } else if (ct == OR_SOLID_NO_SLIP) {
                out = lut.bb[in];
            } else if (ct == OR_SOLID_SLIP) {
                out = (uint8_t)in;
                if (north || south) out = lut.bfx[in];
                if (east || west) out = lut.bfy[in];
            } else {
                out = (uint8_t)in; /* the reference's switch has no default */
            }
            next[cell] = (uint8_t)(out & ((1u << D) - 1u));
        }
    }
    (void)N;
}

/* Forcing column: for every fluid cell (force_x, y) draw a Bernoulli flip and
 * apply the reference's x-direction reversal (src/omp_lattice.cpp:295-300
 * HPP: 2 -> 0, :313-318 FHP: 3 -> 0). */
void oracle_force_column(const oracle_cfg *cfg, const int32_t *types, uint8_t *state,
                         uint64_t t)
{
    if (cfg->force_x < 0 || cfg->force_x >= cfg->W || cfg->force_thr == 0) return;
    const long W = cfg->W, x = cfg->force_x;
    const int west_ch = cfg->model == OR_HPP ? 2 : 3;
    const uint64_t key = lgca_rng_key(cfg->seed, LGCA_STREAM_FORCE, t);
    for (long y = 0; y < cfg->H; ++y) {
        const long cell = y * W + x;
        if (types && types[cell] != OR_FLUID) continue;
        uint64_t u = lgca_rng_draw(key, lgca_rng_index((uint32_t)y, (uint32_t)x)) >> 32;
        if (u >= cfg->force_thr) continue;
        uint8_t s = state[cell];
        if (!BIT(s, 0) && BIT(s, west_ch))
            state[cell] = (uint8_t)((s | 1u) & ~(1u << west_ch));
    }
}

void oracle_run(const oracle_cfg *cfg, const int32_t *types, uint8_t *state, uint8_t *tmp,
                uint64_t t0, int nsteps)
{
    const size_t n = (size_t)cfg->W * (size_t)cfg->H;
    for (int s = 0; s < nsteps; ++s) {
        oracle_force_column(cfg, types, state, t0 + (uint64_t)s);
        oracle_collide_and_propagate(cfg, types, state, tmp, t0 + (uint64_t)s);
        memcpy(state, tmp, n);
    }
}

/* Lattice::init_random, src/lattice.cpp:198-217, with the Bernoulli draws taken
 * from the shared generator and separate probabilities for moving and rest
 * channels. */
void oracle_init_bernoulli(int model, int W, int H, const int32_t *types, uint8_t *state,
                           uint64_t seed, double p_move, double p_rest)
{
    const int D = oracle_num_dir(model);
    uint64_t keys[7], thr[7];
    for (int d = 0; d < D; ++d) {
        keys[d] = lgca_rng_key(seed, LGCA_STREAM_INIT, (uint64_t)d);
        thr[d] = lgca_prob_threshold(d == 6 ? p_rest : p_move);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long y = 0; y < H; ++y) {
        for (long x = 0; x < W; ++x) {
            const long cell = y * (long)W + x;
            uint8_t s = 0;
            if (!types || types[cell] == OR_FLUID) {
                for (int d = 0; d < D; ++d) {
                    uint64_t u = lgca_rng_draw(keys[d], lgca_rng_index((uint32_t)y, (uint32_t)x)) >> 32;
                    if (u < thr[d]) s |= (uint8_t)(1u << d);
                }
            }
            state[cell] = s;
        }
    }
}

void oracle_block_sums(int model, int W, int H, const uint8_t *state, int B, int32_t *N,
                       int32_t *Jx2, int32_t *Jy)
{
    const int Wb = (W + B - 1) / B, Hb = (H + B - 1) / B;
    memset(N, 0, sizeof(int32_t) * (size_t)Wb * Hb);
    memset(Jx2, 0, sizeof(int32_t) * (size_t)Wb * Hb);
    memset(Jy, 0, sizeof(int32_t) * (size_t)Wb * Hb);
    for (long y = 0; y < H; ++y) {
        for (long x = 0; x < W; ++x) {
            const unsigned s = state[y * (long)W + x];
            const long b = (y / B) * Wb + x / B;
            int n = 0, jx2, jy;
            for (int d = 0; d < oracle_num_dir(model); ++d) n += (int)BIT(s, d);
            if (model == OR_HPP) {
                jx2 = 2 * ((int)BIT(s, 0) - (int)BIT(s, 2));
                jy = (int)BIT(s, 1) - (int)BIT(s, 3);
            } else {
                jx2 = 2 * (int)BIT(s, 0) + (int)BIT(s, 1) - (int)BIT(s, 2) - 2 * (int)BIT(s, 3) -
                      (int)BIT(s, 4) + (int)BIT(s, 5);
                jy = (int)BIT(s, 1) + (int)BIT(s, 2) - (int)BIT(s, 4) - (int)BIT(s, 5);
            }
            N[b] += n;
            Jx2[b] += jx2;
            Jy[b] += jy;
        }
    }
}

/* Lattice vectors, src/lgca_models.h:51-52 (HPP) and :246-247 (FHP); the
 * FHP sine is the float value of sin(pi/3) (:236). */
void oracle_cell_post_process(int model, int W, int H, const uint8_t *state,
                              float *cell_density, float *cell_momentum)
{
    const float S = (float)sin(M_PI / 3.0);
    const float vx_h[4] = {1.0f, 0.0f, -1.0f, 0.0f}, vy_h[4] = {0.0f, 1.0f, 0.0f, -1.0f};
    const float vx_f[7] = {1.0f, 0.5f, -0.5f, -1.0f, -0.5f, 0.5f, 0.0f};
    const float vy_f[7] = {0.0f, S, S, 0.0f, -S, -S, 0.0f};
    const float *vx = model == OR_HPP ? vx_h : vx_f, *vy = model == OR_HPP ? vy_h : vy_f;
    const int D = oracle_num_dir(model);
    const long n = (long)W * H;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long cell = 0; cell < n; ++cell) {
        int dens = 0;
        float mx = 0.0f, my = 0.0f;
        for (int d = 0; d < D; ++d) {
            int ns = (int)BIT(state[cell], d);
            dens += ns;
            mx += (float)ns * vx[d];
            my += (float)ns * vy[d];
        }
        cell_density[cell] = (float)dens;
        cell_momentum[2 * cell] = mx;
        cell_momentum[2 * cell + 1] = my;
    }
}

/* src/omp_lattice.cpp:397-454.  The anchor of coarse cell c is the bottom-left
 * cell (2r*cx, 2r*cy); the window loops y = 0..2r, x = 0..2r and keeps a cell
 * when its linear index is inside the lattice and |x_nb - x_anchor| <= r
 * (:434-436), so it is (r+1) wide, (2r+1) tall and clipped at the top.  FP32
 * sums in loop order, then division by the count. */
void oracle_mean_post_process(int W, int H, int r, const float *cell_density,
                              const float *cell_momentum, float *mean_density,
                              float *mean_momentum)
{
    const long Wc = W / (2 * r), Hc = H / (2 * r), n = (long)W * H;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long cc = 0; cc < Wc * Hc; ++cc) {
        const long cell = (cc % Wc) * (2 * r) + (cc / Wc) * (2 * r) * (long)W;
        const long px = cell % W;
        float md = 0.0f, mx = 0.0f, my = 0.0f;
        int cnt = 0;
        for (int y = 0; y <= 2 * r; ++y) {
            for (int x = 0; x <= 2 * r; ++x) {
                const long nb = cell + (long)y * W + x;
                const long pxn = nb % W;
                if (nb < n && labs(pxn - px) <= r) {
                    cnt++;
                    md += cell_density[nb];
                    mx += cell_momentum[2 * nb];
                    my += cell_momentum[2 * nb + 1];
                }
            }
        }
        mean_density[cc] = md / (float)cnt;
        mean_momentum[2 * cc] = mx / (float)cnt;
        mean_momentum[2 * cc + 1] = my / (float)cnt;
    }
}

uint64_t oracle_count_particles(int W, int H, const uint8_t *state)
{
    uint64_t n = 0;
    const long cells = (long)W * H;
    for (long c = 0; c < cells; ++c) n += (uint64_t)__builtin_popcount(state[c]);
    return n;
}

/* src/omp_lattice.cpp:508-557: mean over fluid cells of momentum / density
 * (cells with density <= 1e-6 add nothing but are counted).  The reference
 * sums in FP32 across threads; here the sum is in double in cell order, so
 * results agree to rounding only. */
void oracle_mean_velocity(int W, int H, const int32_t *types, const float *cell_density,
                          const float *cell_momentum, float *ux, float *uy)
{
    double sx = 0.0, sy = 0.0;
    long cnt = 0;
    const long n = (long)W * H;
    for (long c = 0; c < n; ++c) {
        if (types && types[c] != OR_FLUID) continue;
        cnt++;
        float rho = cell_density[c];
        if (rho > 1.0e-06f) {
            sx += (double)(cell_momentum[2 * c] / rho);
            sy += (double)(cell_momentum[2 * c + 1] / rho);
        }
    }
    *ux = (float)(sx / (double)cnt);
    *uy = (float)(sy / (double)cnt);
}

/* OMP_Lattice<M>::apply_body_force, src/omp_lattice.cpp:254-346: draw random
 * cells until `forcing` particles were reverted or 2*num_cells draws were
 * made; only fluid cells are touched.  rand() is replaced by the FSEQ
 * stream: candidate k of call `call` is (draw >> 33) % num_cells. */
unsigned oracle_apply_body_force(int model, int W, int H, const int32_t *types,
                                 uint8_t *state, uint64_t seed, uint64_t call, int forcing,
                                 int bf_dir)
{
    const size_t ncells = (size_t)W * (size_t)H;
    const size_t it_max = 2 * ncells;
    const uint64_t key = lgca_rng_key(seed, LGCA_STREAM_FSEQ, call);
    size_t it = 0;
    unsigned reverted = 0;
    do {
        const size_t cell = (size_t)(int)(lgca_rng_draw(key, it) >> 33) % ncells;
        it++;
        if (types && types[cell] != OR_FLUID) continue;
        uint8_t s = state[cell], o = s;
        if (model == OR_HPP) {
            if (bf_dir == 'x' && !BIT(s, 0) && BIT(s, 2)) {
                o = (uint8_t)((o | 1u) & ~4u);
                reverted++;
            } else if (bf_dir == 'y' && BIT(s, 1) && !BIT(s, 3)) {
                o = (uint8_t)((o & ~2u) | 8u);
                reverted++;
            }
        } else {
            if (bf_dir == 'x' && !BIT(s, 0) && BIT(s, 3)) {
                o = (uint8_t)((o | 1u) & ~8u);
                reverted++;
            } else if (bf_dir == 'y') {
                if (BIT(s, 1) && !BIT(s, 5)) {
                    o = (uint8_t)((o & ~2u) | 32u);
                    reverted++;
                }
                if (BIT(s, 2) && !BIT(s, 4)) {
                    o = (uint8_t)((o & ~4u) | 16u);
                    reverted++;
                }
            }
        }
        state[cell] = o;
    } while (reverted < (unsigned)forcing && it < it_max);
    return reverted;
}
