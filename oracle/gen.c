/*
 * gen.c -- synthetic tensors for the CPU reference arm.
 *
 * TEST INFRASTRUCTURE ONLY.  A plain restatement of the synthetic generator
 * the benchmark's workloads come from, so that the CPU reference arm can draw
 * its sample without loading the product library:
 *
 *   draw d picks index a of the cell from u = hash(seed, 11, d, a) through the
 *   inverse CDF of Zipf(s_a) over the axis (uniform when s_a = 0); the
 *   entries are the first nnz distinct cells in draw order; a cell's value is
 *   the ground-truth CP model (factors gt_std * N(0,1) from hash(seed, 21+a,
 *   i*R + r)) plus noise_std * N(0,1) from hash(seed, 31, cell), or, with no
 *   ground truth, exp(N(0,1)) from hash(seed, 32, cell) rescaled to [0, 1]
 *   by the largest value; it is a train entry when hash(seed, 41, cell) <
 *   train_frac.  Train and test entries keep draw order.
 *
 * Because the entries are the first distinct cells in draw order, a draw of
 * nnz = M cells is the first M cells of any larger draw with the same seed
 * and shape (values included, except that log-normal values are rescaled by
 * the sample's own largest value).
 *
 * Build with -ffp-contract=off: values are (a*b)*c summed in rank order.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t g_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static uint64_t g_hash4(uint64_t seed, uint64_t a, uint64_t b, uint64_t c)
{
    return g_mix64(g_mix64(g_mix64(seed ^ g_mix64(a)) ^ b) ^ c);
}

static double g_unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

static double g_normal(uint64_t h1, uint64_t h2)
{
    double u1 = g_unit(h1), u2 = g_unit(h2);
    if (u1 < 1e-300)
        u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

typedef struct {
    int n;
    double s;
    double *cdf;
} g_zipf;

static int g_zipf_init(g_zipf *z, int n, double s)
{
    z->n = n;
    z->s = s;
    z->cdf = NULL;
    if (s <= 0)
        return 0;
    z->cdf = (double *)malloc(sizeof(double) * (size_t)n);
    if (!z->cdf)
        return -1;
    double acc = 0;
    for (int i = 0; i < n; i++) {
        acc += pow((double)(i + 1), -s);
        z->cdf[i] = acc;
    }
    for (int i = 0; i < n; i++)
        z->cdf[i] /= acc;
    return 0;
}

/* first index whose cdf is >= u (lower bound), at most n - 1 */
static int g_zipf_sample(const g_zipf *z, double u)
{
    if (z->s <= 0) {
        int k = (int)(u * z->n);
        return k < z->n - 1 ? k : z->n - 1;
    }
    int lo = 0, hi = z->n;
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (z->cdf[mid] < u)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo < z->n - 1 ? lo : z->n - 1;
}

int orc_gen_tensor(int I, int J, int K, int64_t nnz, const double *zipf_s, int R, double gt_std,
                   double noise_std, double train_frac, uint64_t seed, int32_t **txyz, double **tval,
                   int64_t *ntr, int32_t **sxyz, double **sval, int64_t *nte)
{
    if (I <= 0 || J <= 0 || K <= 0 || nnz < 0 || (double)nnz > 0.5 * (double)I * (double)J * (double)K)
        return 1;
    const int dims[3] = {I, J, K};
    g_zipf z[3];
    for (int a = 0; a < 3; a++)
        if (g_zipf_init(&z[a], dims[a], zipf_s[a]))
            return 3;
    const uint64_t JK = (uint64_t)J * (uint64_t)K;
    uint64_t cap = 1024;
    while (cap < (uint64_t)nnz * 2 + 16)
        cap <<= 1;
    uint64_t *table = (uint64_t *)malloc(sizeof(uint64_t) * cap);
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(nnz > 0 ? nnz : 1));
    if (!table || !keys)
        return 3;
    memset(table, 0xff, sizeof(uint64_t) * cap);
    int64_t nk = 0;
    for (uint64_t d = 0; nk < nnz; d++) {
        if (d > (uint64_t)nnz * 1000 + (1ULL << 26)) {
            free(table);
            free(keys);
            return 8;
        }
        uint64_t x = (uint64_t)g_zipf_sample(&z[0], g_unit(g_hash4(seed, 11, d, 0)));
        uint64_t y = (uint64_t)g_zipf_sample(&z[1], g_unit(g_hash4(seed, 11, d, 1)));
        uint64_t w = (uint64_t)g_zipf_sample(&z[2], g_unit(g_hash4(seed, 11, d, 2)));
        uint64_t k = x * JK + y * (uint64_t)K + w;
        uint64_t h = g_mix64(k) & (cap - 1);
        while (table[h] != ~0ULL && table[h] != k)
            h = (h + 1) & (cap - 1);
        if (table[h] == ~0ULL) {
            table[h] = k;
            keys[nk++] = k;
        }
    }
    free(table);
    for (int a = 0; a < 3; a++)
        free(z[a].cdf);
    double *gt[3] = {NULL, NULL, NULL};
    for (int a = 0; a < 3 && R > 0; a++) {
        int64_t m = (int64_t)dims[a] * R;
        gt[a] = (double *)malloc(sizeof(double) * (size_t)m);
        if (!gt[a])
            return 3;
        for (int64_t i = 0; i < m; i++)
            gt[a][i] = gt_std * g_normal(g_hash4(seed, 21 + a, (uint64_t)i, 0), g_hash4(seed, 21 + a, (uint64_t)i, 1));
    }
    int32_t *xyz = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(nk > 0 ? nk : 1));
    double *val = (double *)malloc(sizeof(double) * (size_t)(nk > 0 ? nk : 1));
    unsigned char *is_train = (unsigned char *)malloc((size_t)(nk > 0 ? nk : 1));
    if (!xyz || !val || !is_train)
        return 3;
    double mx = 0;
    for (int64_t i = 0; i < nk; i++) {
        uint64_t k = keys[i];
        int32_t x = (int32_t)(k / JK), y = (int32_t)((k / (uint64_t)K) % (uint64_t)J), w = (int32_t)(k % (uint64_t)K);
        xyz[3 * i] = x;
        xyz[3 * i + 1] = y;
        xyz[3 * i + 2] = w;
        double v;
        if (R > 0) {
            v = 0;
            for (int r = 0; r < R; r++)
                v += gt[0][(size_t)x * R + r] * gt[1][(size_t)y * R + r] * gt[2][(size_t)w * R + r];
            v += noise_std * g_normal(g_hash4(seed, 31, k, 0), g_hash4(seed, 31, k, 1));
        } else {
            v = exp(g_normal(g_hash4(seed, 32, k, 0), g_hash4(seed, 32, k, 1)));
            if (v > mx)
                mx = v;
        }
        val[i] = v;
        is_train[i] = g_unit(g_hash4(seed, 41, k, 0)) < train_frac;
    }
    if (R <= 0 && nk > 0)
        for (int64_t i = 0; i < nk; i++)
            val[i] /= mx;
    for (int a = 0; a < 3; a++)
        free(gt[a]);
    free(keys);
    int64_t na = 0, nb = 0;
    for (int64_t i = 0; i < nk; i++) {
        if (is_train[i])
            na++;
        else
            nb++;
    }
    *txyz = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(na > 0 ? na : 1));
    *tval = (double *)malloc(sizeof(double) * (size_t)(na > 0 ? na : 1));
    *sxyz = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(nb > 0 ? nb : 1));
    *sval = (double *)malloc(sizeof(double) * (size_t)(nb > 0 ? nb : 1));
    if (!*txyz || !*tval || !*sxyz || !*sval)
        return 3;
    int64_t ia = 0, ib = 0;
    for (int64_t i = 0; i < nk; i++) {
        if (is_train[i]) {
            memcpy(*txyz + 3 * ia, xyz + 3 * i, 12);
            (*tval)[ia++] = val[i];
        } else {
            memcpy(*sxyz + 3 * ib, xyz + 3 * i, 12);
            (*sval)[ib++] = val[i];
        }
    }
    free(xyz);
    free(val);
    free(is_train);
    *ntr = na;
    *nte = nb;
    return 0;
}

void orc_gen_free(void *p) { free(p); }
