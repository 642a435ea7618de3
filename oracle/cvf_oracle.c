/*
 * CPU oracle for the CVF bulk-water NPT Monte Carlo step -- TEST INFRASTRUCTURE ONLY.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this file's
 * library; the GPU engine never links it.
 *
 * It restates the reference program SOURCE/gpu_water3D.cu (lcoronas/CVFBulkWater) in the
 * reference's own layout (byte per arm variable, s[arm*N+cell], eta[arm*N+cell], one cube
 * state per 2x2x2 cube indexed as in GW:3203) and drives it with the engine's Philox streams.
 * Every function names the reference lines it follows ("GW" = SOURCE/gpu_water3D.cu,
 * "CB" = SOURCE/chessboard.h).
 *
 * The random-number plumbing of the reference (MT19937, xorshift1024*, cuRAND XORWOW
 * buffers; GW:2833-2864, GW:2954-2976) is replaced by counter-based Philox4x32-10
 * (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11):
 *   key     = (seed & 0xffffffff, seed >> 32)
 *   counter = (site, move counter, stream tag, replica)
 * so that every accept/reject decision is an integer comparison reproducible on the GPU.
 *
 * Compile with -ffp-contract=off: the FP64 volume move must round exactly like the GPU.
 */
#include "cvf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- constants */
/* Model constants, float literals as in GW:57-64. */
#define J_HB_F 0.5f
#define J_SIG_F 0.08f
#define V_HB_F 0.6f
#define ARMS 6
#define Q 6
#define EDGES 12
#define NSOL 9

/* Stream tags (counter word 2). */
#define ST_SWEEP 0x01u
#define ST_SWEEP_REFINE 0x02u
#define ST_CUBE 0x03u
#define ST_VOLUME 0x04u
#define ST_SW_FLIP 0x05u
#define ST_INIT_SIGMA 0x06u
#define ST_INIT_CUBE 0x07u
#define ST_INIT_ORDER 0x08u
#define ST_CUBE_REFINE 0x09u
#define ST_SW_BOND 0x10u        /* + 0..2 */
#define ST_SW_BOND_REFINE 0x18u /* + 0..2 */
#define ST_WOLFF_POKE 0x0Au     /* counter (lo P, hi P, tag): seed site and shift of poke P */
#define ST_WOLFF_SHIFT 0x0Bu    /* retry kind of the shift draw */
#define ST_WOLFF_BOND 0x20u     /* + l/4, counter (owner cell, lo P, tag | hi P << 8) */
#define ST_RETRY(kind, k) (0x1000u | ((uint32_t)(kind) << 8) | (uint32_t)(k))

/* ------------------------------------------------------------------ Philox */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        if (round) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct oracle {
    int L;
    int64_t N;
    float T, P, Rc;
    double beta, Jeff;
    uint32_t key[2], replica;
    uint32_t ctr[4]; /* sweep, cube, volume, sw */
    uint8_t *s, *eta, *cube;
    int32_t* label;
    double r_cell, V, E_vdw;
    int n_shells;
    float dist[512];
    int freq[512];
    uint64_t thr_sweep[33], thr_cube[9], thr_sw[2];
    int nthreads;
    int chess;    /* Flag_chessboard: 1 cube moves, 0 the nhb<=4 mode */
    int wolff;    /* cluster steps are Wolff steps (GW:2199-2357) instead of Swendsen-Wang */
    uint64_t wpoke;                 /* Wolff pokes so far (the poke counter P) */
    int64_t w_pokes, w_sum, w_max;  /* the last Wolff step: pokes, summed and largest size */
    uint8_t* nhb; /* Flag_chessboard = 0: dev_nhb of GW:1974-2007, one byte per cell */
};

static void rng(const oracle_t* o, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t out[4])
{
    uint32_t ctr[4] = {c0, c1, c2, o->replica};
    oracle_philox4x32_10(ctr, o->key, out);
}

/* Uniform integer in [0, n) by Lemire's multiply-shift with exact rejection: try the
 * given words in order, then word 0 of the retry stream ST_RETRY(kind, k), k = 0..255. */
static uint32_t draw_below(const oracle_t* o, uint32_t n, const uint32_t* words, int nwords,
                           uint32_t c0, uint32_t c1, uint32_t kind)
{
    uint32_t thr = (uint32_t)(0u - n) % n;
    uint64_t m = 0;
    for (int i = 0; i < nwords; ++i) {
        m = (uint64_t)words[i] * n;
        if ((uint32_t)m >= thr) return (uint32_t)(m >> 32);
    }
    for (uint32_t k = 0; k < 256; ++k) {
        uint32_t r[4];
        rng(o, c0, c1, ST_RETRY(kind, k), r);
        m = (uint64_t)r[0] * n;
        if ((uint32_t)m >= thr) return (uint32_t)(m >> 32);
    }
    return (uint32_t)(m >> 32);
}

static uint64_t thr_from_p(double p)
{
    if (p >= 1.0) return 1ull << 32;
    if (!(p > 0.0)) return 0;
    double t = floor(p * 4294967296.0 + 0.5);
    if (t >= 4294967296.0) return 1ull << 32;
    return (uint64_t)t;
}

static double u53(uint32_t lo, uint32_t hi)
{
    uint64_t b = ((((uint64_t)hi) << 32) | lo) >> 11;
    return (double)b * (1.0 / 9007199254740992.0);
}

/* -------------------------------------------------------- own exp and log */
static double bits_to_d(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t d_to_bits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }

#define LN2_HI 0.6931467056274414        /* ln 2 with the low 32 mantissa bits cleared */
#define LN2_LO 4.7493250390316726e-07    /* ln 2 - LN2_HI */
#define INV_LN2 1.4426950408889634

/* exp(x): k = round(x/ln2), r = x - k ln2 (two-part), Taylor series of e^r to r^13,
 * scaled by 2^k built from its exponent bits. Results below 2^-1022 are flushed to 0. */
double oracle_exp(double x)
{
    if (x != x) return x;
    if (x > 709.78) return HUGE_VAL;
    if (x < -708.3) return 0.0;
    double kd = floor(x * INV_LN2 + 0.5);
    double r = (x - kd * LN2_HI) - kd * LN2_LO;
    double p = 1.6059043836821613e-10;
    p = p * r + 2.08767569878681e-09;
    p = p * r + 2.505210838544172e-08;
    p = p * r + 2.755731922398589e-07;
    p = p * r + 2.7557319223985893e-06;
    p = p * r + 2.48015873015873e-05;
    p = p * r + 0.0001984126984126984;
    p = p * r + 0.001388888888888889;
    p = p * r + 0.008333333333333333;
    p = p * r + 0.041666666666666664;
    p = p * r + 0.16666666666666666;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    int k = (int)kd;
    return p * bits_to_d((uint64_t)(k + 1023) << 52);
}

/* log(x): x = m 2^e with m in [1/sqrt2, sqrt2), log m = 2 atanh(s), s = (m-1)/(m+1),
 * odd series to s^25; result e*ln2 + log m with the two-part ln 2. */
double oracle_log(double x)
{
    if (x != x) return x;
    if (x < 0.0) return NAN;
    if (x == 0.0) return -HUGE_VAL;
    if (x > 1.7976931348623157e308) return x;
    uint64_t b = d_to_bits(x);
    int e = (int)((b >> 52) & 0x7ff);
    if (e == 0) { /* subnormal */
        b = d_to_bits(x * 18014398509481984.0); /* 2^54 */
        e = (int)((b >> 52) & 0x7ff) - 54;
    }
    double m = bits_to_d((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
    e -= 1023;
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double z = s * s;
    double q = 0.04;
    q = q * z + 0.043478260869565216;
    q = q * z + 0.047619047619047616;
    q = q * z + 0.05263157894736842;
    q = q * z + 0.058823529411764705;
    q = q * z + 0.06666666666666667;
    q = q * z + 0.07692307692307693;
    q = q * z + 0.09090909090909091;
    q = q * z + 0.1111111111111111;
    q = q * z + 0.14285714285714285;
    q = q * z + 0.2;
    q = q * z + 0.3333333333333333;
    q = q * z + 1.0;
    double lm = (2.0 * s) * q;
    double ed = (double)e;
    return ed * LN2_HI + (ed * LN2_LO + lm);
}

/* ------------------------------------------------------------ geometry */
static inline int64_t cell_of(int L, int x, int y, int z) { return (int64_t)x + (int64_t)L * (y + (int64_t)L * z); }

/* neighbour of cell along arm a: 0 x+, 1 x-, 2 y+, 3 y-, 4 z+, 5 z- (GW:1936-1962) */
static inline int64_t neighbour(int L, int64_t cell, int a)
{
    int x = (int)(cell % L), y = (int)((cell / L) % L), z = (int)(cell / ((int64_t)L * L));
    switch (a) {
    case 0: x = (x + 1) % L; break;
    case 1: x = (x - 1 + L) % L; break;
    case 2: y = (y + 1) % L; break;
    case 3: y = (y - 1 + L) % L; break;
    case 4: z = (z + 1) % L; break;
    default: z = (z - 1 + L) % L; break;
    }
    return cell_of(L, x, y, z);
}

/* Cube edges in the reference's numbering (CB:41-53): direction (0 x, 1 y, 2 z) and start
 * vertex as offset bits dx | dy<<1 | dz<<2 (v1=0, v2=1, v3=2, v4=4, v5=7, v6=6, v7=5, v8=3). */
static const int edge_dir[EDGES] = {0, 1, 2, 2, 1, 2, 0, 1, 0, 0, 1, 2};
static const int edge_start[EDGES] = {0, 0, 0, 1, 1, 2, 2, 4, 4, 6, 5, 3};
/* Inactive edges of the nine solutions (CB:155-208). */
static const int sol_off[NSOL][4] = {{2, 3, 6, 9}, {2, 3, 5, 11}, {0, 6, 8, 9},  {0, 5, 8, 11}, {1, 3, 7, 11},
                                     {1, 4, 7, 10}, {2, 4, 5, 10}, {1, 4, 8, 9}, {0, 6, 7, 10}};
static int sol_active(int s, int e)
{
    for (int i = 0; i < 4; ++i)
        if (sol_off[s][i] == e) return 0;
    return 1;
}

/* cube storage index of the reference (GW:3203) for an origin with all-even or all-odd coords */
static inline int64_t cube_index(int L, int x, int y, int z)
{
    return (int64_t)(x / 2) + (int64_t)(L / 2) * (y / 2) + (int64_t)(L * L / 4) * z;
}

static void edge_cells(int L, int x0, int y0, int z0, int e, int64_t* v0, int64_t* v1)
{
    int st = edge_start[e], d = edge_dir[e];
    int x = (x0 + (st & 1)) % L, y = (y0 + ((st >> 1) & 1)) % L, z = (z0 + ((st >> 2) & 1)) % L;
    *v0 = cell_of(L, x, y, z);
    *v1 = neighbour(L, *v0, 2 * d);
}

/* write eta of both endpoints of the 12 edges from the cube state (GW:3447-3464) */
static void cube_write_eta(oracle_t* o, int x0, int y0, int z0, int state)
{
    for (int e = 0; e < EDGES; ++e) {
        int64_t v0, v1;
        edge_cells(o->L, x0, y0, z0, e, &v0, &v1);
        int d = edge_dir[e];
        uint8_t a = (uint8_t)sol_active(state, e);
        o->eta[(int64_t)(2 * d) * o->N + v0] = a;
        o->eta[(int64_t)(2 * d + 1) * o->N + v1] = a;
    }
}

/* Enumerate cube origins: all-even or all-odd coordinates (GW:3189-3197). */
static inline int cube_origin_from_index(int L, int64_t i, int* x, int* y, int* z)
{
    /* i in [0, N/4): z = i / (L*L/4), rem -> (x/2, y/2) */
    int64_t per_plane = (int64_t)L * L / 4;
    int zz = (int)(i / per_plane);
    int64_t rem = i % per_plane;
    int hx = (int)(rem % (L / 2)), hy = (int)(rem / (L / 2));
    int odd = zz & 1;
    *x = 2 * hx + odd;
    *y = 2 * hy + odd;
    *z = zz;
    return 1;
}

/* ------------------------------------------------------------ vdW shells */
/* GW:865-932 with distance_PBC GW:1323-1337 */
int oracle_distances(int L, float Rc, float* dist, int* freq, int cap)
{
    int n = 0;
    int64_t N = (int64_t)L * L * L;
    for (int64_t j = 1; j < N; ++j) {
        int x2 = (int)(j % L), y2 = (int)((j / L) % L), z2 = (int)(j / ((int64_t)L * L));
        int dx = abs(0 - x2), dy = abs(0 - y2), dz = abs(0 - z2);
        if (dx > L / 2) dx = L - dx;
        if (dy > L / 2) dy = L - dy;
        if (dz > L / 2) dz = L - dz;
        float d = (float)sqrt((double)(dx * dx + dy * dy + dz * dz));
        if (d < Rc) {
            int found = 0;
            for (int k = 0; k < n; ++k)
                if (d == dist[k]) {
                    freq[k]++;
                    found = 1;
                    break;
                }
            if (!found) {
                if (n >= cap) return -1;
                dist[n] = d;
                freq[n] = 1;
                n++;
            }
        }
    }
    for (int k = 0; k < n; ++k) {
        freq[k] /= 2;
        freq[k] *= (int)N;
    }
    return n;
}

/* GW:1784-1805 */
double oracle_evdw(const oracle_t* o, double r)
{
    double tmp = 1.0 / (double)o->Rc;
    tmp = tmp * tmp * tmp;
    double att = tmp * tmp;
    double rep = att * att;
    double shift = rep - att;
    double ret = 0.0;
    for (int i = 0; i < o->n_shells; ++i) {
        double rd = r * (double)o->dist[i];
        if (rd < (double)o->Rc) {
            tmp = 1.0 / rd;
            tmp = tmp * tmp * tmp;
            att = tmp * tmp;
            rep = att * att;
            ret += (double)o->freq[i] * (rep - att - shift);
        }
    }
    return ret;
}

/* ------------------------------------------------------------ create */
static void build_tables(oracle_t* o)
{
    double Js = (double)J_SIG_F;
    for (int dhb = -1; dhb <= 1; ++dhb)
        for (int dns = -5; dns <= 5; ++dns) {
            double dE = -o->Jeff * (double)dhb - Js * (double)dns;
            o->thr_sweep[(dhb + 1) * 11 + dns + 5] = thr_from_p(exp(-o->beta * dE));
        }
    for (int dhb = -4; dhb <= 4; ++dhb) {
        double dE = -o->Jeff * (double)dhb - Js * 0.0;
        o->thr_cube[dhb + 4] = thr_from_p(exp(-o->beta * dE));
    }
    /* GW:992-993 */
    o->thr_sw[0] = thr_from_p(1.0 - exp(-o->beta * fabs(o->Jeff)));
    o->thr_sw[1] = thr_from_p(1.0 - exp(-o->beta * fabs(Js)));
}

static void random_cubes(oracle_t* o)
{
    int64_t ncubes = o->N / 4;
    for (int64_t i = 0; i < ncubes; ++i) {
        int x, y, z;
        cube_origin_from_index(o->L, i, &x, &y, &z);
        uint32_t cid = (uint32_t)cell_of(o->L, x, y, z);
        uint32_t r[4];
        rng(o, cid, 0, ST_INIT_CUBE, r);
        int st = (int)draw_below(o, NSOL, r, 4, cid, 0, ST_INIT_CUBE);
        o->cube[i] = (uint8_t)st;
        cube_write_eta(o, x, y, z, st);
    }
}

static void nhb_init(oracle_t* o);

oracle_t* oracle_create(int L, float T, float P, int64_t seed, float Rc, uint32_t replica, int start)
{
    return oracle_create_mode(L, T, P, seed, Rc, replica, start, 1);
}

/* flag_chessboard = 0: every eta is 1 (GW:721-724), no cube moves, and the bond count per cell
 * (GW:841-862) drives the nhb<=4 dynamics. */
oracle_t* oracle_create_mode(int L, float T, float P, int64_t seed, float Rc, uint32_t replica, int start,
                             int flag_chessboard)
{
    if (L < 4 || (L & 1)) return NULL;
    oracle_t* o = (oracle_t*)calloc(1, sizeof(oracle_t));
    o->L = L;
    o->N = (int64_t)L * L * L;
    o->T = T;
    o->P = P;
    o->Rc = Rc;
    o->beta = 1. / T;                                  /* GW:388 */
    o->Jeff = (double)(float)(J_HB_F - P * V_HB_F);    /* GW:391, float expression */
    o->key[0] = (uint32_t)((uint64_t)seed & 0xffffffffu);
    o->key[1] = (uint32_t)((uint64_t)seed >> 32);
    o->replica = replica;
    o->nthreads = 1;
    o->s = (uint8_t*)calloc((size_t)(ARMS * o->N), 1);
    o->eta = (uint8_t*)calloc((size_t)(ARMS * o->N), 1);
    o->cube = (uint8_t*)calloc((size_t)(o->N / 4), 1);
    o->label = (int32_t*)calloc((size_t)(ARMS * o->N), sizeof(int32_t));
    o->n_shells = oracle_distances(L, Rc, o->dist, o->freq, 512);
    o->r_cell = 1.0001;                                   /* GW:150 */
    o->V = (double)o->N * o->r_cell * o->r_cell * o->r_cell; /* GW:481 */
    o->E_vdw = oracle_evdw(o, o->r_cell);
    build_tables(o);
    if (start == 0) { /* disordered: GW:812-817 */
        for (int64_t c = 0; c < o->N; ++c) {
            uint32_t r[4];
            rng(o, (uint32_t)c, 0, ST_INIT_SIGMA, r);
            uint32_t d = draw_below(o, 46656u, r, 4, (uint32_t)c, 0, ST_INIT_SIGMA);
            for (int a = 0; a < ARMS; ++a) {
                o->s[a * o->N + c] = (uint8_t)(d % 6);
                d /= 6;
            }
        }
        random_cubes(o);
    } else if (start == 2) { /* ordered: GW:819-825 */
        uint32_t r[4];
        rng(o, 0, 0, ST_INIT_ORDER, r);
        uint8_t s0 = (uint8_t)draw_below(o, 6, r, 4, 0, 0, ST_INIT_ORDER);
        memset(o->s, s0, (size_t)(ARMS * o->N));
        random_cubes(o);
    } else {
        random_cubes(o);
    }
    o->chess = flag_chessboard != 0;
    o->nhb = (uint8_t*)calloc((size_t)o->N, 1);
    if (!o->chess) {
        memset(o->eta, 1, (size_t)(ARMS * o->N));
        nhb_init(o);
    }
    return o;
}

void oracle_destroy(oracle_t* o)
{
    if (!o) return;
    free(o->s);
    free(o->eta);
    free(o->cube);
    free(o->label);
    free(o->nhb);
    free(o);
}

void oracle_set_threads(oracle_t* o, int n) { o->nthreads = n > 0 ? n : 1; }

/* ------------------------------------------------------------ config */
/* GW:730-811 (read) and GW:3314-3371 (infer cube state from eta) */
int oracle_set_config(oracle_t* o, const int32_t* c12, int64_t n_cells)
{
    if (n_cells != o->N) return -1;
    for (int64_t c = 0; c < o->N; ++c)
        for (int a = 0; a < ARMS; ++a) {
            int sv = c12[c * 12 + a], ev = c12[c * 12 + 6 + a];
            if (sv < 0 || sv > 5 || ev < 0 || ev > 1) return -2;
            o->s[a * o->N + c] = (uint8_t)sv;
            o->eta[a * o->N + c] = (uint8_t)ev;
        }
    if (!o->chess) { /* GW:791-806 infers cube states only with Flag_chessboard = 1 */
        nhb_init(o);
        return 0;
    }
    int L = o->L;
    int64_t ncubes = o->N / 4;
    for (int64_t i = 0; i < ncubes; ++i) {
        int x, y, z;
        cube_origin_from_index(L, i, &x, &y, &z);
        int xp = (x + 1) % L, yp = (y + 1) % L, zp = (z + 1) % L;
        int64_t v1 = cell_of(L, x, y, z), v2 = cell_of(L, xp, y, z), v3 = cell_of(L, x, yp, z);
        int64_t v6 = cell_of(L, x, yp, zp), v7 = cell_of(L, xp, y, zp), v8 = cell_of(L, xp, yp, z);
        const uint8_t* eta = o->eta;
        int64_t N = o->N;
        int st;
        if (eta[0 * N + v1] == 0) {
            if (eta[0 * N + v6] == 0) st = 2;
            else if (eta[4 * N + v3] == 0) st = 3;
            else st = 8;
        } else if (eta[2 * N + v1] == 0) {
            if (eta[4 * N + v2] == 0) st = 4;
            else if (eta[2 * N + v7] == 0) st = 5;
            else st = 7;
        } else {
            if (eta[0 * N + v3] == 0) st = 0;
            else if (eta[4 * N + v8] == 0) st = 1;
            else st = 6;
        }
        o->cube[i] = (uint8_t)st;
    }
    /* the first cube move of the reference rewrites every eta from the inferred states */
    for (int64_t i = 0; i < ncubes; ++i) {
        int x, y, z;
        cube_origin_from_index(L, i, &x, &y, &z);
        cube_write_eta(o, x, y, z, o->cube[i]);
    }
    return 0;
}

int oracle_get_config(const oracle_t* o, int32_t* c12, int64_t n_cells)
{
    if (n_cells != o->N) return -1;
    for (int64_t c = 0; c < o->N; ++c)
        for (int a = 0; a < ARMS; ++a) {
            c12[c * 12 + a] = o->s[a * o->N + c];
            c12[c * 12 + 6 + a] = o->eta[a * o->N + c];
        }
    return 0;
}

/* even cubes indexed (x/2) + (L/2)(y/2) + (L/2)^2 (z/2) for origins (2a,2b,2c); odd cubes the
 * same for origins (2a+1,2b+1,2c+1). */
void oracle_get_cubes(const oracle_t* o, uint8_t* ev, uint8_t* od)
{
    int L = o->L, H = L / 2;
    int64_t ncubes = o->N / 4;
    for (int64_t i = 0; i < ncubes; ++i) {
        int x, y, z;
        cube_origin_from_index(L, i, &x, &y, &z);
        int64_t k = (int64_t)(x / 2) + (int64_t)H * (y / 2) + (int64_t)H * H * (z / 2);
        if (z & 1) od[k] = o->cube[i];
        else ev[k] = o->cube[i];
    }
}

/* ------------------------------------------------------------ moves */
/* Cube (chessboard) Metropolis move: GW:3374-3466, CPU twin CB:326-478. All cubes at once:
 * cubes share no edge and sigma is fixed, so the update order does not matter.
 * Random numbers: the cubes of one parity are grouped by four consecutive along x (origins
 * x = 2*hx + parity, hx = 4g .. 4g+3, same y and z; the last group of a row holds fewer when
 * L/2 is not a multiple of 4). Group g draws one Philox block at the cell id of its first cube's
 * origin: words 0 and 3 (then the retry streams of ST_CUBE) give an exact uniform in [0, 9^4)
 * whose base-9 digit k (most significant first) is the proposed state of cube hx = 4g + k; the
 * acceptance uniform of cube k is the 32-bit U with high half (k & 1) of word 1 + (k >> 1) and
 * low half at the same position of the refinement block (ST_CUBE_REFINE), drawn only when the
 * high half equals T >> 16. */
void oracle_cube_move(oracle_t* o)
{
    int L = o->L;
    int64_t N = o->N, ncubes = N / 4;
    uint32_t t = o->ctr[1];
    static const uint32_t pow9[4] = {729, 81, 9, 1};
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
    for (int64_t i = 0; i < ncubes; ++i) {
        int x, y, z;
        cube_origin_from_index(L, i, &x, &y, &z);
        int hx = x / 2, k = hx & 3, odd = x & 1;
        uint32_t gid = (uint32_t)cell_of(L, 2 * (hx - k) + odd, y, z);
        uint32_t r[4];
        rng(o, gid, t, ST_CUBE, r);
        uint32_t pw[2] = {r[0], r[3]};
        uint32_t d = draw_below(o, 6561u, pw, 2, gid, t, ST_CUBE);
        int nw = (int)((d / pow9[k]) % 9);
        int old = o->cube[i];
        int dhb = 0;
        for (int e = 0; e < EDGES; ++e) {
            int64_t v0, v1;
            edge_cells(L, x, y, z, e, &v0, &v1);
            int dd = edge_dir[e];
            int same = o->s[(int64_t)(2 * dd) * N + v0] == o->s[(int64_t)(2 * dd + 1) * N + v1];
            dhb += (sol_active(nw, e) - sol_active(old, e)) * same;
        }
        uint64_t T = o->thr_cube[dhb + 4];
        uint32_t hU = (r[1 + (k >> 1)] >> (16 * (k & 1))) & 0xffffu;
        int acc;
        if ((uint64_t)hU != (T >> 16)) {
            acc = (uint64_t)hU < (T >> 16);
        } else {
            uint32_t rf[4];
            rng(o, gid, t, ST_CUBE_REFINE, rf);
            uint32_t lU = (rf[1 + (k >> 1)] >> (16 * (k & 1))) & 0xffffu;
            acc = ((((uint64_t)hU) << 16) | lU) < T;
        }
        if (!acc) nw = old;
        o->cube[i] = (uint8_t)nw;
        cube_write_eta(o, x, y, z, nw);
    }
    o->ctr[1]++;
}

/* NPT volume move: GW:1740-1781 */
void oracle_volume_move(oracle_t* o)
{
    uint32_t t = o->ctr[2];
    uint32_t r[4];
    rng(o, 0, t, ST_VOLUME, r);
    double u1 = u53(r[0], r[1]);
    double trial = o->r_cell + 0.01 * 2 * (u1 - 0.5);
    for (uint32_t k = 1; trial < 0.0 && k < 64; ++k) { /* LJ_InfiniteBarrier = 0 (GW:119) */
        uint32_t rr[4];
        rng(o, k, t, ST_VOLUME, rr);
        u1 = u53(rr[0], rr[1]);
        trial = o->r_cell + 0.01 * 2 * (u1 - 0.5);
    }
    int L = o->L;
    double tV = trial * trial * trial * (double)L * (double)L * (double)L;
    double dV = tV - o->V;
    double tE = oracle_evdw(o, trial);
    double NT = (double)((float)o->N * o->T);
    double dE = (tE - o->E_vdw) - NT * oracle_log(tV / o->V);
    double u2 = u53(r[2], r[3]);
    if (u2 < oracle_exp(-o->beta * (dE + (double)o->P * dV))) {
        o->r_cell = trial;
        o->V = tV;
        o->E_vdw = tE;
    }
    o->ctr[2]++;
}

/* Metropolis update of all six sigma arms of one cell, arms in order 0..5 (the engine's
 * checkerboard sweep). Proposal of arm a: base-6 digit a, most significant first, of the
 * uniform d in [0, 46656) drawn from word 0. Energy change as in GW:1964-1996 (chessboard branch):
 *   dN_hb = eta_a [delta(new, s'_opp) - delta(old, s'_opp)],
 *   dN_s  = sum_{b != a} [delta(new, s_b) - delta(old, s_b)],
 * accepted iff U < T[dN_hb, dN_s] with U = 32-bit uniform whose high half is chunk a of
 * words 1..3 of the sweep block and whose low half is chunk a of the refinement block. */
static void sweep_cell(oracle_t* o, int64_t cell, uint32_t t)
{
    int64_t N = o->N;
    uint32_t r[4], rf[4];
    int have_rf = 0;
    rng(o, (uint32_t)cell, t, ST_SWEEP, r);
    static const uint32_t pow6[ARMS] = {7776, 1296, 216, 36, 6, 1};
    uint32_t d = draw_below(o, 46656u, r, 1, (uint32_t)cell, t, ST_SWEEP);
    for (int a = 0; a < ARMS; ++a) {
        int nw = (int)((d / pow6[a]) % 6);
        int old = o->s[a * N + cell];
        if (nw == old) continue;
        int nb = o->s[(int64_t)(a ^ 1) * N + neighbour(o->L, cell, a)];
        int dhb = o->eta[a * N + cell] * ((nw == nb) - (old == nb));
        int dns = 0;
        for (int b = 0; b < ARMS; ++b) {
            if (b == a) continue;
            int sb = o->s[b * N + cell];
            dns += (nw == sb) - (old == sb);
        }
        uint64_t T = o->thr_sweep[(dhb + 1) * 11 + dns + 5];
        uint32_t hU = (r[1 + a / 2] >> (16 * (a & 1))) & 0xffffu;
        int acc;
        if (hU != (uint32_t)(T >> 16)) {
            acc = hU < (T >> 16);
        } else {
            if (!have_rf) {
                rng(o, (uint32_t)cell, t, ST_SWEEP_REFINE, rf);
                have_rf = 1;
            }
            uint32_t lU = (rf[a / 2] >> (16 * (a & 1))) & 0xffffu;
            acc = ((((uint64_t)hU) << 16) | lU) < T;
        }
        if (acc) o->s[a * N + cell] = (uint8_t)nw;
    }
}

/* GW:841-862: bonds of each cell whose two arms agree, counted only where eta = 1. */
static void nhb_init(oracle_t* o)
{
    int64_t N = o->N;
    for (int64_t c = 0; c < N; ++c) {
        int acc = 0;
        for (int a = 0; a < ARMS; ++a)
            acc += o->eta[a * N + c] * (o->s[a * N + c] == o->s[(int64_t)(a ^ 1) * N + neighbour(o->L, c, a)]);
        o->nhb[c] = (uint8_t)acc;
    }
}

/* Flag_chessboard = 0 (GW:1964-2007, non-chessboard branch): arm a of one cell with the same
 * random numbers as the checkerboard sweep (proposal digit a of word 0, acceptance uniform chunk
 * a), and the hydrogen-bond term theta(nhb_i + d <= 4) theta(nhb_j + d <= 4) delta(new, s') minus
 * theta(nhb_i <= 4) theta(nhb_j <= 4) delta(old, s'), with d = delta(new, s') - delta(old, s').
 * On acceptance both cells' counts move by d, as bytes. */
static void sweep_cell_arm_nhb(oracle_t* o, int64_t cell, int a, uint32_t t)
{
    int64_t N = o->N;
    uint32_t r[4];
    rng(o, (uint32_t)cell, t, ST_SWEEP, r);
    static const uint32_t pow6[ARMS] = {7776, 1296, 216, 36, 6, 1};
    uint32_t d = draw_below(o, 46656u, r, 1, (uint32_t)cell, t, ST_SWEEP);
    int nw = (int)((d / pow6[a]) % 6);
    int old = o->s[a * N + cell];
    if (nw == old) return;
    int64_t j = neighbour(o->L, cell, a);
    int nb = o->s[(int64_t)(a ^ 1) * N + j];
    int dn = (nw == nb) - (old == nb);
    int ni = o->nhb[cell], nj = o->nhb[j];
    int hbn = (ni + dn <= 4) * (nj + dn <= 4) * (nw == nb);
    int hbo = (ni <= 4) * (nj <= 4) * (old == nb);
    int dhb = hbn - hbo;
    int dns = 0;
    for (int b = 0; b < ARMS; ++b) {
        if (b == a) continue;
        int sb = o->s[b * N + cell];
        dns += (nw == sb) - (old == sb);
    }
    uint64_t T = o->thr_sweep[(dhb + 1) * 11 + dns + 5];
    uint32_t hU = (r[1 + a / 2] >> (16 * (a & 1))) & 0xffffu;
    int acc;
    if (hU != (uint32_t)(T >> 16)) {
        acc = hU < (T >> 16);
    } else {
        uint32_t rf[4];
        rng(o, (uint32_t)cell, t, ST_SWEEP_REFINE, rf);
        uint32_t lU = (rf[a / 2] >> (16 * (a & 1))) & 0xffffu;
        acc = ((((uint64_t)hU) << 16) | lU) < T;
    }
    if (acc) {
        o->s[a * N + cell] = (uint8_t)nw;
        o->nhb[cell] = (uint8_t)(ni + dn);
        o->nhb[j] = (uint8_t)(nj + dn);
    }
}

void oracle_sweep(oracle_t* o)
{
    int L = o->L;
    uint32_t t = o->ctr[0];
    if (!o->chess) {
        /* colour 0 arms 0..5, then colour 1 arms 0..5: in one (colour, arm) pass no two cells
         * share a neighbour along the arm, so the cells are independent */
        for (int colour = 0; colour < 2; ++colour)
            for (int a = 0; a < ARMS; ++a)
                for (int64_t zy = 0; zy < (int64_t)L * L; ++zy) {
                    int y = (int)(zy % L), z = (int)(zy / L);
                    for (int x = (y + z + colour) & 1; x < L; x += 2) sweep_cell_arm_nhb(o, cell_of(L, x, y, z), a, t);
                }
        o->ctr[0]++;
        return;
    }
    for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
        for (int64_t zy = 0; zy < (int64_t)L * L; ++zy) {
            int y = (int)(zy % L), z = (int)(zy / L);
            int x0 = (y + z + colour) & 1;
            for (int x = x0; x < L; x += 2) sweep_cell(o, cell_of(L, x, y, z), t);
        }
    }
    o->ctr[0]++;
}

/* ------------------------------------------------------------ Swendsen-Wang */
static int32_t uf_find(int32_t* p, int32_t a)
{
    int32_t r = a;
    while (p[r] != r) r = p[r];
    while (p[a] != r) {
        int32_t nx = p[a];
        p[a] = r;
        a = nx;
    }
    return r;
}
static void uf_union(int32_t* p, int32_t a, int32_t b)
{
    int32_t ra = uf_find(p, a), rb = uf_find(p, b);
    if (ra == rb) return;
    if (ra < rb) p[rb] = ra;
    else p[ra] = rb;
}

/* Bond decision of link l of a cell from its three bond blocks w[0..11]: U < T for the 32-bit
 * uniform U whose high half is half (l & 1) of word l >> 1 and whose low half sits at the same
 * position of the cell's refinement blocks (ST_SW_BOND_REFINE + 0..2), drawn only when the high
 * half equals T >> 16. */
static int sw_link(const oracle_t* o, const uint32_t* w, int l, uint64_t T, uint32_t c, uint32_t t)
{
    uint32_t hU = (w[l >> 1] >> (16 * (l & 1))) & 0xffffu;
    if ((uint64_t)hU != (T >> 16)) return (uint64_t)hU < (T >> 16);
    uint32_t rf[4];
    rng(o, c, t, ST_SW_BOND_REFINE + (uint32_t)(l >> 3), rf);
    uint32_t lU = (rf[(l >> 1) & 3] >> (16 * (l & 1))) & 0xffffu;
    return ((((uint64_t)hU) << 16) | lU) < T;
}

/* Bonds GW:2383-2438 (18 links per cell: x+, y+, z+ hydrogen-bond links then the 15
 * intra-cell pairs a<b in row-major order), components over the 6N arm sites labelled by
 * their minimum site id (the fixed point of GW:2440-2529), cluster shift GW:2531-2542.
 * Random numbers per cell and SW step: three Philox blocks (ST_SW_BOND + 0..2, words w[0..11]);
 * link l uses the 16-bit halves described at sw_link; words 9, 10 (then the retry streams of
 * ST_SW_FLIP) give an exact uniform d in [0, 6^6) whose base-6 digit a (most significant first)
 * is the shift of the cluster whose root is the cell's arm site a. */
void oracle_sw_step(oracle_t* o)
{
    int L = o->L;
    int64_t N = o->N, NS = ARMS * N;
    uint32_t t = o->ctr[3];
    int32_t* p = o->label;
    static const uint32_t pow6[ARMS] = {7776, 1296, 216, 36, 6, 1};
    uint8_t* shift = (uint8_t*)malloc(NS > 0 ? (size_t)NS : 1);
    for (int64_t i = 0; i < NS; ++i) p[i] = (int32_t)i;
    for (int64_t c = 0; c < N; ++c) {
        uint32_t w[12];
        for (uint32_t j = 0; j < 3; ++j) rng(o, (uint32_t)c, t, ST_SW_BOND + j, &w[4 * j]);
        for (int d = 0; d < 3; ++d) {
            int64_t A = (int64_t)(2 * d) * N + c;
            int64_t B = (int64_t)(2 * d + 1) * N + neighbour(L, c, 2 * d);
            int bond = 0;
            if (o->Jeff > 0)
                bond = o->eta[A] && o->s[A] == o->s[B] && sw_link(o, w, d, o->thr_sw[0], (uint32_t)c, t);
            else if (o->Jeff < 0)
                bond = o->s[A] != o->s[B] && sw_link(o, w, d, o->thr_sw[0], (uint32_t)c, t);
            if (bond) uf_union(p, (int32_t)A, (int32_t)B);
        }
        int l = 3;
        for (int a = 0; a < ARMS - 1; ++a)
            for (int b = a + 1; b < ARMS; ++b, ++l)
                if (o->s[a * N + c] == o->s[b * N + c] && sw_link(o, w, l, o->thr_sw[1], (uint32_t)c, t))
                    uf_union(p, (int32_t)(a * N + c), (int32_t)(b * N + c));
        uint32_t dsh = draw_below(o, 46656u, &w[9], 2, (uint32_t)c, t, ST_SW_FLIP);
        for (int a = 0; a < ARMS; ++a) shift[a * N + c] = (uint8_t)((dsh / pow6[a]) % 6);
    }
    for (int64_t i = 0; i < NS; ++i) p[i] = uf_find(p, (int32_t)i);
    for (int64_t i = 0; i < NS; ++i) o->s[i] = (uint8_t)((o->s[i] + shift[p[i]]) % Q);
    free(shift);
    o->ctr[3]++;
}

/* ------------------------------------------------------------ Wolff */
/* Bond of link l of owner cell c in Wolff poke P: U < T with the 32-bit uniform U = word l & 3 of
 * the block ST_WOLFF_BOND + l/4 at counter (c, lo P, tag | hi P << 8). */
static int wolff_link(const oracle_t* o, int64_t c, int l, uint64_t P)
{
    uint32_t r[4];
    rng(o, (uint32_t)c, (uint32_t)P, (ST_WOLFF_BOND + (uint32_t)(l >> 2)) | ((uint32_t)(P >> 32) << 8), r);
    return (uint64_t)r[l & 3] < o->thr_sw[l < 3 ? 0 : 1];
}

/* Link index of the intra-cell pair (a, b), a < b, in row-major order after the three
 * hydrogen-bond links (the numbering of the Swendsen-Wang links). */
static int pair_link(int a, int b)
{
    static const int base[5] = {0, 5, 9, 12, 14};
    return 3 + base[a] + (b - a - 1);
}

/* GW:2199-2357, cluster_step: pokes until the clusters flipped add up to 6N sites. Poke P takes
 * a seed site in [0, 6N) and a shift in 1..5 (block ST_WOLFF_POKE at (lo P, hi P): words 0-2 and
 * 3, exact draws), grows the seed's cluster over the bonds of the Swendsen-Wang step (the
 * hydrogen-bond link of arm 2d of a cell with arm 2d+1 of its +d neighbour: eta and equal sigma
 * for Jeff > 0, different sigma for Jeff < 0; the 15 intra-cell pairs: equal sigma), each bond
 * decided once per poke from its own uniform, and shifts every site of it by the shift (mod 6).
 * The cluster is the seed's connected component in the bond graph of the poke, so it does not
 * depend on the order of the search (the reference's recursion order picks which random number
 * tests which bond). */
void oracle_wolff_step(oracle_t* o)
{
    int L = o->L;
    int64_t N = o->N, NS = ARMS * N;
    int64_t* stack = (int64_t*)malloc((size_t)(NS > 0 ? NS : 1) * sizeof(int64_t));
    uint8_t* mark = (uint8_t*)calloc((size_t)(NS > 0 ? NS : 1), 1);
    int64_t done = 0, pokes = 0, maxs = 0;
    while (done < NS) {
        uint64_t P = o->wpoke++;
        uint32_t r[4];
        rng(o, (uint32_t)P, (uint32_t)(P >> 32), ST_WOLFF_POKE, r);
        int64_t seed = draw_below(o, (uint32_t)NS, r, 3, (uint32_t)P, (uint32_t)(P >> 32), ST_WOLFF_POKE);
        uint32_t shift = 1u + draw_below(o, 5u, &r[3], 1, (uint32_t)P, (uint32_t)(P >> 32), ST_WOLFF_SHIFT);
        int64_t n = 0, head = 0;
        stack[n++] = seed;
        mark[seed] = 1;
        while (head < n) {
            int64_t site = stack[head++];
            int a = (int)(site / N);
            int64_t c = site % N;
            uint8_t sa = o->s[site];
            for (int b = 0; b < ARMS; ++b) {
                if (b == a) continue;
                int64_t sb = (int64_t)b * N + c;
                if (mark[sb] || o->s[sb] != sa) continue;
                if (!wolff_link(o, c, pair_link(a < b ? a : b, a < b ? b : a), P)) continue;
                mark[sb] = 1;
                stack[n++] = sb;
            }
            int d = a >> 1;
            int64_t owner = (a & 1) ? neighbour(L, c, a) : c;
            int64_t other = (a & 1) ? (int64_t)(2 * d) * N + owner : (int64_t)(2 * d + 1) * N + neighbour(L, c, a);
            if (mark[other]) continue;
            int cond = 0;
            if (o->Jeff > 0) cond = o->eta[(int64_t)(2 * d) * N + owner] && o->s[other] == sa;
            else if (o->Jeff < 0) cond = o->s[other] != sa;
            if (cond && wolff_link(o, owner, d, P)) {
                mark[other] = 1;
                stack[n++] = other;
            }
        }
        for (int64_t i = 0; i < n; ++i) {
            o->s[stack[i]] = (uint8_t)((o->s[stack[i]] + shift) % Q);
            mark[stack[i]] = 0;
        }
        done += n;
        ++pokes;
        if (n > maxs) maxs = n;
    }
    o->w_pokes = pokes;
    o->w_sum = done;
    o->w_max = maxs;
    free(stack);
    free(mark);
    o->ctr[3]++;
}

void oracle_set_wolff(oracle_t* o, int on) { o->wolff = on != 0; }

void oracle_wolff_stats(const oracle_t* o, int64_t out[4])
{
    out[0] = o->w_pokes;
    out[1] = o->w_sum;
    out[2] = o->w_max;
    out[3] = (int64_t)o->wpoke;
}

static void cluster_step(oracle_t* o)
{
    if (o->wolff) oracle_wolff_step(o);
    else oracle_sw_step(o);
}

void oracle_step(oracle_t* o, int nmet, int ncl)
{
    if (!o->chess) { /* GW:1348-1384: no cube move; SW leaves the bond counts stale (GW:2531-2542) */
        oracle_volume_move(o);
        for (int j = 0; j < nmet; ++j) oracle_sweep(o);
        for (int j = 0; j < ncl; ++j) cluster_step(o);
        return;
    }
    oracle_cube_move(o);
    oracle_volume_move(o);
    for (int j = 0; j < nmet; ++j) oracle_sweep(o);
    for (int j = 0; j < ncl; ++j) cluster_step(o);
}

/* ------------------------------------------------------------ observables */
/* GW:2014-2160 (chessboard branch) */
void oracle_measure(const oracle_t* o, oracle_obs_t* out)
{
    int L = o->L;
    int64_t N = o->N;
    int64_t hb2 = 0, ns = 0;
    if (!o->chess) {
        /* GW:2064-2099: bonds in typewriter order (cell, then x+, y+, z+), each counted for both
         * cells while both have fewer than NHBMAX = 4; hb2 = sum of the counts = 2 N_hb */
        uint8_t* cnt = (uint8_t*)calloc((size_t)N, 1);
        for (int64_t c = 0; c < N; ++c)
            for (int d = 0; d < 3; ++d) {
                int64_t nb = neighbour(L, c, 2 * d);
                if (o->s[(int64_t)(2 * d) * N + c] == o->s[(int64_t)(2 * d + 1) * N + nb] && cnt[c] < 4 && cnt[nb] < 4) {
                    cnt[c]++;
                    cnt[nb]++;
                    hb2 += 2;
                }
            }
        free(cnt);
        for (int64_t c = 0; c < N; ++c)
            for (int a = 0; a < ARMS - 1; ++a)
                for (int b = a + 1; b < ARMS; ++b) ns += o->s[a * N + c] == o->s[b * N + c];
    } else {
#pragma omp parallel for schedule(static) reduction(+ : hb2, ns) num_threads(o->nthreads)
        for (int64_t c = 0; c < N; ++c) {
            for (int d = 0; d < 3; ++d) {
                int64_t nb = neighbour(L, c, 2 * d);
                if (o->s[(int64_t)(2 * d) * N + c] == o->s[(int64_t)(2 * d + 1) * N + nb])
                    hb2 += o->eta[(int64_t)(2 * d) * N + c] + o->eta[(int64_t)(2 * d + 1) * N + nb];
            }
            for (int a = 0; a < ARMS - 1; ++a)
                for (int b = a + 1; b < ARMS; ++b) ns += o->s[a * N + c] == o->s[b * N + c];
        }
    }
    out->n_hb2 = hb2;
    out->n_sigma = ns;
    out->r_cell = o->r_cell;
    out->volume = o->V;
    out->e_vdw = oracle_evdw(o, o->r_cell);
    out->n_hb = 0.5 * (double)hb2;
    out->energy = (out->e_vdw + (-(double)J_HB_F) * out->n_hb) + (-(double)J_SIG_F) * (double)ns;
    out->v_total = (double)N * o->r_cell * o->r_cell * o->r_cell + (double)V_HB_F * out->n_hb;
    out->enthalpy = out->energy + (double)o->P * out->v_total;
    out->m = (double)ns / ((double)N * 15.0);
}

/* GW:2677-2780 */
void oracle_cluster_stats(const oracle_t* o, oracle_cstats_t* out)
{
    int L = o->L;
    int64_t N = o->N, NS = ARMS * N;
    int32_t* size = (int32_t*)calloc((size_t)NS, sizeof(int32_t));
    for (int64_t i = 0; i < NS; ++i) size[o->label[i]]++;
    int64_t largest = 0, second = 0, ncl = 0, sum = 0, sum2 = 0, sum2w = 0;
    int32_t* cand = (int32_t*)malloc((size_t)NS * sizeof(int32_t));
    int64_t ncand = 0;
    for (int64_t i = 0; i < NS; ++i) {
        int64_t sz = size[i];
        if (sz == 0) {
            cand[i] = -1;
            continue;
        }
        ncl++;
        sum += sz;
        sum2 += sz * sz;
        sum2w += (int32_t)(uint32_t)((uint64_t)sz * (uint64_t)sz);
        if (sz > largest) {
            second = largest;
            largest = sz;
        } else if (sz > second) {
            second = sz;
        }
        cand[i] = (sz >= 2 * L) ? (int32_t)(ncand++) : -1;
    }
    int64_t nperc = 0;
    if (ncand) {
        uint8_t* cov = (uint8_t*)calloc((size_t)(ncand * 3 * L), 1);
        for (int64_t i = 0; i < NS; ++i) {
            int32_t k = cand[o->label[i]];
            if (k < 0) continue;
            int64_t c = i % N;
            int x = (int)(c % L), y = (int)((c / L) % L), z = (int)(c / ((int64_t)L * L));
            cov[(int64_t)k * 3 * L + x] = 1;
            cov[(int64_t)k * 3 * L + L + y] = 1;
            cov[(int64_t)k * 3 * L + 2 * L + z] = 1;
        }
        for (int64_t k = 0; k < ncand; ++k) {
            int full[3] = {1, 1, 1};
            for (int ax = 0; ax < 3; ++ax)
                for (int j = 0; j < L; ++j)
                    if (!cov[k * 3 * L + ax * L + j]) {
                        full[ax] = 0;
                        break;
                    }
            nperc += (full[0] || full[1] || full[2]);
        }
        free(cov);
    }
    free(cand);
    free(size);
    out->largest = largest;
    out->second = second;
    out->n_percolating = nperc;
    out->n_clusters = ncl;
    out->sum_size = sum;
    out->sum_size2 = sum2;
    out->sum_size2_wrap32 = sum2w;
}

void oracle_get_labels(const oracle_t* o, int32_t* labels)
{
    memcpy(labels, o->label, (size_t)(ARMS * o->N) * sizeof(int32_t));
}

void oracle_get_state(const oracle_t* o, double* r, double* v, double* e, uint32_t ctr[4])
{
    *r = o->r_cell;
    *v = o->V;
    *e = o->E_vdw;
    memcpy(ctr, o->ctr, sizeof(o->ctr));
}

void oracle_set_state(oracle_t* o, double r, double v, const uint32_t ctr[4])
{
    o->r_cell = r;
    o->V = v;
    o->E_vdw = oracle_evdw(o, r);
    memcpy(o->ctr, ctr, sizeof(o->ctr));
}

void oracle_get_thresholds(const oracle_t* o, uint64_t* s33, uint64_t* c9, uint64_t* sw2)
{
    memcpy(s33, o->thr_sweep, sizeof(o->thr_sweep));
    memcpy(c9, o->thr_cube, sizeof(o->thr_cube));
    memcpy(sw2, o->thr_sw, sizeof(o->thr_sw));
}

void oracle_get_nhb(const oracle_t* o, uint8_t* nhb) { memcpy(nhb, o->nhb, (size_t)o->N); }
