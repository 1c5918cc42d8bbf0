/*
 * CPU oracle for the BSC block-sorting stage (forward BWT + primary index,
 * inverse BWT).  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the
 * CPU-baseline leg of the benchmark use it as the checker.  Nothing in the
 * product path links or calls this file.
 *
 * What it restates.  qz reaches the block sorter through libbsc's
 * bsc_compress / bsc_decompress (crates/qz-lib/src/compression/bsc.rs:91-125,
 * call sites bsc.rs:172-183 and bsc.rs:401-433).  libbsc's BWT stage
 * (libbsc/bwt/bwt.cpp, which wraps libsais) is NOT in the reference tree: it is
 * compiled from an un-vendored third_party/libbsc at an unpinned HEAD
 * (crates/qz-lib/build.rs:56-75, README.md:900).  This file therefore restates
 * the published algorithms in its own code:
 *
 *   - suffix sorting by induced sorting (SA-IS, Nong, Zhang & Chan 2009), with
 *     an implicit end sentinel smaller than every byte;
 *   - a brute-force suffix sort (direct comparison) as an independent check,
 *     and prefix doubling (Manber & Myers 1993) as a second one for sizes
 *     brute force cannot reach;
 *   - the libsais BWT output convention (libsais is libbsc's CPU sorter,
 *     build.rs:62): U[0] = T[n-1], then the last column of the sorted matrix
 *     with the sentinel row dropped, and the primary index = 1 + the rank of
 *     the whole string among the n non-empty suffixes;
 *   - auxiliary indexes at a power-of-two sampling rate r, as libsais_bwt_aux
 *     defines them: I[k] = 1 + rank of suffix k*r (so I[0] is the primary
 *     index);
 *   - the inverse BWT by LF-mapping.
 *
 * Parity status: UNPINNED against libbsc.  No reference test pins BWT bytes or
 * the primary index (bsc.rs:438-499 only round-trips), and libbsc cannot be
 * built here.  The convention is pinned against the brute-force definition and
 * textbook known answers instead; PRIMARY_INDEX_OFFSET is the one constant to
 * flip if libbsc's stored index turns out to differ.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PRIMARY_INDEX_OFFSET 1

#define ORACLE_NO_ERROR 0
#define ORACLE_BAD_PARAMETER -1
#define ORACLE_NOT_ENOUGH_MEMORY -2
#define ORACLE_DATA_CORRUPT -6

/* ------------------------------------------------------------------------ */
/* SA-IS over an integer string whose last symbol is a unique minimum (0).   */
/* ------------------------------------------------------------------------ */

static void bucket_bounds(const int32_t *s, int32_t n, int32_t K, int32_t *bkt, int want_end)
{
    memset(bkt, 0, (size_t)K * sizeof(int32_t));
    for (int32_t i = 0; i < n; ++i) bkt[s[i]]++;
    int32_t run = 0;
    for (int32_t c = 0; c < K; ++c) {
        int32_t cnt = bkt[c];
        run += cnt;
        bkt[c] = want_end ? run : run - cnt;
    }
}

#define STYPE(i) ((stype[(i) >> 3] >> ((i) & 7)) & 1)
#define IS_LMS(i) ((i) > 0 && STYPE(i) && !STYPE((i) - 1))

static void induce(const int32_t *s, int32_t *SA, int32_t n, int32_t K, int32_t *bkt,
                   const uint8_t *stype)
{
    /* L-type suffixes, left to right from bucket heads */
    bucket_bounds(s, n, K, bkt, 0);
    for (int32_t i = 0; i < n; ++i) {
        int32_t j = SA[i] - 1;
        if (SA[i] > 0 && !STYPE(j)) SA[bkt[s[j]]++] = j;
    }
    /* S-type suffixes, right to left from bucket tails */
    bucket_bounds(s, n, K, bkt, 1);
    for (int32_t i = n - 1; i >= 0; --i) {
        int32_t j = SA[i] - 1;
        if (SA[i] > 0 && STYPE(j)) SA[--bkt[s[j]]] = j;
    }
}

/* returns 0 or a negative error */
static int sais_int(const int32_t *s, int32_t *SA, int32_t n, int32_t K)
{
    if (n == 1) { SA[0] = 0; return 0; }
    uint8_t *stype = (uint8_t *)calloc(((size_t)n + 7) / 8, 1);
    int32_t *bkt = (int32_t *)malloc((size_t)K * sizeof(int32_t));
    if (!stype || !bkt) { free(stype); free(bkt); return ORACLE_NOT_ENOUGH_MEMORY; }

    /* classify: last symbol (the sentinel) is S-type */
    stype[(n - 1) >> 3] |= (uint8_t)(1u << ((n - 1) & 7));
    for (int32_t i = n - 2; i >= 0; --i) {
        int st = s[i] < s[i + 1] || (s[i] == s[i + 1] && STYPE(i + 1));
        if (st) stype[i >> 3] |= (uint8_t)(1u << (i & 7));
    }

    /* stage 1: sort LMS substrings by one induced pass */
    for (int32_t i = 0; i < n; ++i) SA[i] = -1;
    bucket_bounds(s, n, K, bkt, 1);
    for (int32_t i = 1; i < n; ++i)
        if (IS_LMS(i)) SA[--bkt[s[i]]] = i;
    induce(s, SA, n, K, bkt, stype);

    /* gather the sorted LMS positions at the front */
    int32_t n1 = 0;
    for (int32_t i = 0; i < n; ++i)
        if (IS_LMS(SA[i])) SA[n1++] = SA[i];

    /* name LMS substrings; names land in SA[n1 + pos/2] */
    for (int32_t i = n1; i < n; ++i) SA[i] = -1;
    int32_t names = 0, prev = -1;
    for (int32_t i = 0; i < n1; ++i) {
        int32_t pos = SA[i];
        int differ = 0;
        if (prev < 0) {
            differ = 1;
        } else {
            for (int32_t d = 0;; ++d) {
                if (pos + d >= n || prev + d >= n || s[pos + d] != s[prev + d] ||
                    STYPE(pos + d) != STYPE(prev + d)) {
                    differ = 1;
                    break;
                }
                if (d > 0 && (IS_LMS(pos + d) || IS_LMS(prev + d))) break;
            }
        }
        if (differ) { names++; prev = pos; }
        SA[n1 + (pos >> 1)] = names - 1;
    }
    /* pack the reduced string into the tail of SA */
    for (int32_t i = n - 1, j = n - 1; i >= n1; --i)
        if (SA[i] >= 0) SA[j--] = SA[i];
    int32_t *s1 = SA + n - n1;

    /* stage 2: sort the reduced string */
    if (names < n1) {
        int rc = sais_int(s1, SA, n1, names);
        if (rc) { free(stype); free(bkt); return rc; }
    } else {
        for (int32_t i = 0; i < n1; ++i) SA[s1[i]] = i;
    }

    /* stage 3: induce the full order from the sorted LMS suffixes */
    for (int32_t i = 1, j = 0; i < n; ++i)
        if (IS_LMS(i)) s1[j++] = i;
    for (int32_t i = 0; i < n1; ++i) SA[i] = s1[SA[i]];
    for (int32_t i = n1; i < n; ++i) SA[i] = -1;
    bucket_bounds(s, n, K, bkt, 1);
    for (int32_t i = n1 - 1; i >= 0; --i) {
        int32_t j = SA[i];
        SA[i] = -1;
        SA[--bkt[s[j]]] = j;
    }
    induce(s, SA, n, K, bkt, stype);
    free(stype);
    free(bkt);
    return 0;
}

/*
 * Suffix array of T[0..n) with an implicit end sentinel that is smaller than
 * every byte (so a suffix that is a prefix of another sorts first).
 * SA receives the n non-empty suffixes in order.
 */
int oracle_suffix_array(const uint8_t *T, int32_t *SA, int32_t n)
{
    if (n < 0 || (n > 0 && (!T || !SA))) return ORACLE_BAD_PARAMETER;
    if (n == 0) return 0;
    int32_t *s = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    int32_t *sa = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    if (!s || !sa) { free(s); free(sa); return ORACLE_NOT_ENOUGH_MEMORY; }
    for (int32_t i = 0; i < n; ++i) s[i] = (int32_t)T[i] + 1;
    s[n] = 0;
    int rc = sais_int(s, sa, n + 1, 257);
    if (rc == 0) memcpy(SA, sa + 1, (size_t)n * sizeof(int32_t)); /* sa[0] == n */
    free(s);
    free(sa);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Brute force: direct suffix comparison (small n only).                     */
/* ------------------------------------------------------------------------ */

static const uint8_t *g_bf_text;
static int32_t g_bf_n;

static int bf_cmp(const void *a, const void *b)
{
    int32_t i = *(const int32_t *)a, j = *(const int32_t *)b;
    int32_t li = g_bf_n - i, lj = g_bf_n - j;
    int32_t m = li < lj ? li : lj;
    int c = memcmp(g_bf_text + i, g_bf_text + j, (size_t)m);
    if (c) return c;
    return li < lj ? -1 : (li > lj ? 1 : 0);
}

/* not thread-safe (qsort has no context argument in C99); tests call it serially */
int oracle_suffix_array_bruteforce(const uint8_t *T, int32_t *SA, int32_t n)
{
    if (n < 0) return ORACLE_BAD_PARAMETER;
    for (int32_t i = 0; i < n; ++i) SA[i] = i;
    g_bf_text = T;
    g_bf_n = n;
    qsort(SA, (size_t)n, sizeof(int32_t), bf_cmp);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Prefix doubling (Manber & Myers 1993), a second independent sorter for    */
/* sizes brute force cannot reach.                                           */
/* ------------------------------------------------------------------------ */

/*
 * Round h sorts the suffixes by their first 2h symbols: the pair (rank of
 * suffix i, rank of suffix i+h), where a suffix that ends inside the first h
 * symbols gets the smallest second key (the end sentinel).  Each round is two
 * stable counting sorts (second key, then first key) and a dense re-ranking;
 * it stops once every rank is distinct.  O(n log n) time, 4n ints of memory.
 */
int oracle_suffix_array_doubling(const uint8_t *T, int32_t *SA, int32_t n)
{
    if (n < 0 || (n > 0 && (!T || !SA))) return ORACLE_BAD_PARAMETER;
    if (n == 0) return 0;
    size_t cn = (size_t)(n > 256 ? n : 256) + 2;
    int32_t *rk = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *nrk = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *tmp = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *cnt = (int32_t *)malloc(cn * sizeof(int32_t));
    if (!rk || !nrk || !tmp || !cnt) {
        free(rk); free(nrk); free(tmp); free(cnt);
        return ORACLE_NOT_ENOUGH_MEMORY;
    }
    for (int32_t i = 0; i < n; ++i) rk[i] = T[i];
    int32_t K = 256; /* ranks are in [0, K) */
    for (int64_t h = 1;; h <<= 1) {
        /* second key: 0 when suffix i ends within h symbols, else 1 + rank */
#define KEY2(i) ((int64_t)(i) + h < n ? rk[(i) + h] + 1 : 0)
        memset(cnt, 0, ((size_t)K + 1) * sizeof(int32_t));
        for (int32_t i = 0; i < n; ++i) cnt[KEY2(i)]++;
        for (int32_t c = 0, run = 0; c <= K; ++c) { int32_t t = cnt[c]; cnt[c] = run; run += t; }
        for (int32_t i = 0; i < n; ++i) tmp[cnt[KEY2(i)]++] = i;
        memset(cnt, 0, (size_t)K * sizeof(int32_t));
        for (int32_t i = 0; i < n; ++i) cnt[rk[i]]++;
        for (int32_t c = 0, run = 0; c < K; ++c) { int32_t t = cnt[c]; cnt[c] = run; run += t; }
        for (int32_t j = 0; j < n; ++j) { int32_t i = tmp[j]; SA[cnt[rk[i]]++] = i; }
        int32_t r = 0;
        nrk[SA[0]] = 0;
        for (int32_t j = 1; j < n; ++j) {
            int32_t a = SA[j - 1], b = SA[j];
            if (rk[a] != rk[b] || KEY2(a) != KEY2(b)) ++r;
            nrk[b] = r;
        }
#undef KEY2
        memcpy(rk, nrk, (size_t)n * sizeof(int32_t));
        K = r + 1;
        if (K == n || h >= n) break;
    }
    free(rk); free(nrk); free(tmp); free(cnt);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Forward BWT with the libsais output convention.                           */
/* ------------------------------------------------------------------------ */

/*
 * U[0..n) receives the BWT; returns the primary index (>= 1 for n >= 1, 0 for
 * n == 0) or a negative error.  If r > 0 (a power of two) and I != NULL,
 * I[0..(n-1)/r] receives the auxiliary indexes I[k] = 1 + rank(suffix k*r),
 * with I[0] equal to the primary index.
 */
int oracle_bwt_from_sa(const uint8_t *T, const int32_t *SA, uint8_t *U, int32_t n, int32_t r,
                       int32_t *I)
{
    if (n == 0) return 0;
    int32_t primary = -1;
    U[0] = T[n - 1];
    int32_t out = 1;
    for (int32_t j = 0; j < n; ++j) {
        int32_t p = SA[j];
        if (p == 0) {
            primary = j + PRIMARY_INDEX_OFFSET;
        } else {
            U[out++] = T[p - 1];
        }
        if (r > 0 && I && (p & (r - 1)) == 0) I[p / r] = j + PRIMARY_INDEX_OFFSET;
    }
    return primary;
}

int oracle_bwt_encode(const uint8_t *T, uint8_t *U, int32_t n, int32_t r, int32_t *I)
{
    if (n < 0 || (n > 0 && (!T || !U))) return ORACLE_BAD_PARAMETER;
    if (r < 0 || (r > 0 && (r & (r - 1)) != 0)) return ORACLE_BAD_PARAMETER;
    if (n == 0) return 0;
    int32_t *SA = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!SA) return ORACLE_NOT_ENOUGH_MEMORY;
    int rc = oracle_suffix_array(T, SA, n);
    if (rc == 0) rc = oracle_bwt_from_sa(T, SA, U, n, r, I);
    free(SA);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Inverse BWT by LF-mapping.                                                */
/* ------------------------------------------------------------------------ */

/*
 * Rows of the sentinel matrix are numbered 0..n; row 0 is the empty suffix and
 * row `index` holds the sentinel in the last column.  U lists the last column
 * with that row dropped.  Walking LF from row 0 yields T from the back.
 * Returns 0, or ORACLE_DATA_CORRUPT when the index is out of range or the LF
 * chain does not close after exactly n steps.
 */
int oracle_bwt_decode(const uint8_t *U, uint8_t *T, int32_t n, int32_t index)
{
    if (n < 0 || (n > 0 && (!U || !T))) return ORACLE_BAD_PARAMETER;
    if (n == 0) return 0;
    int32_t p = index - PRIMARY_INDEX_OFFSET + 1; /* sentinel row in [1, n] */
    if (p < 1 || p > n) return ORACLE_DATA_CORRUPT;
    int64_t C[257];
    memset(C, 0, sizeof(C));
    for (int32_t i = 0; i < n; ++i) C[U[i] + 1]++;
    C[0] = 1; /* row 0 of the first column is the sentinel */
    for (int c = 1; c <= 256; ++c) C[c] += C[c - 1];
    /* C[c] now = 1 + number of symbols < c, shifted: use C[c] for symbol c */
    int32_t *LF = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    if (!LF) return ORACLE_NOT_ENOUGH_MEMORY;
    int64_t next[256];
    for (int c = 0; c < 256; ++c) next[c] = C[c];
    for (int32_t row = 0; row <= n; ++row) {
        if (row == p) { LF[row] = 0; continue; }
        uint8_t c = U[row < p ? row : row - 1];
        LF[row] = (int32_t)next[c]++;
    }
    int32_t row = 0;
    for (int32_t k = n - 1; k >= 0; --k) {
        if (row == p) { free(LF); return ORACLE_DATA_CORRUPT; }
        T[k] = U[row < p ? row : row - 1];
        row = LF[row];
    }
    int ok = row == p;
    free(LF);
    return ok ? 0 : ORACLE_DATA_CORRUPT;
}

/* ------------------------------------------------------------------------ */
/* Many blocks over host threads (one block per thread at a time, the model */
/* qz uses with rayon: bsc.rs:285-288, compression/mod.rs:402-404).          */
/* ------------------------------------------------------------------------ */

typedef struct {
    int direction; /* 0 forward, 1 inverse */
    int32_t nblocks;
    const uint8_t *const *in;
    uint8_t *const *out;
    const int32_t *n;
    int32_t *index; /* forward: written; inverse: read */
    int32_t *status;
    int32_t next;
    pthread_mutex_t lock;
} batch_job;

static void *batch_worker(void *arg)
{
    batch_job *job = (batch_job *)arg;
    for (;;) {
        pthread_mutex_lock(&job->lock);
        int32_t b = job->next++;
        pthread_mutex_unlock(&job->lock);
        if (b >= job->nblocks) break;
        if (job->direction == 0) {
            int rc = oracle_bwt_encode(job->in[b], job->out[b], job->n[b], 0, NULL);
            job->index[b] = rc;
            job->status[b] = rc < 0 ? rc : 0;
        } else {
            job->status[b] = oracle_bwt_decode(job->in[b], job->out[b], job->n[b], job->index[b]);
        }
    }
    return NULL;
}

int oracle_bwt_batch(int direction, int32_t nblocks, const uint8_t *const *in, uint8_t *const *out,
                     const int32_t *n, int32_t *index, int32_t *status, int32_t nthreads)
{
    if (nblocks < 0 || nthreads < 1) return ORACLE_BAD_PARAMETER;
    batch_job job;
    job.direction = direction;
    job.nblocks = nblocks;
    job.in = in;
    job.out = out;
    job.n = n;
    job.index = index;
    job.status = status;
    job.next = 0;
    pthread_mutex_init(&job.lock, NULL);
    if (nthreads > nblocks) nthreads = nblocks > 0 ? nblocks : 1;
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    if (!th) return ORACLE_NOT_ENOUGH_MEMORY;
    for (int32_t t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, batch_worker, &job);
    for (int32_t t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&job.lock);
    for (int32_t b = 0; b < nblocks; ++b)
        if (status[b] < 0) return status[b];
    return 0;
}
