/*
 * glint_query_oracle.c -- CPU restatement of contact-trace queries over the
 * key-value store: a breadth-first expansion over meetings.
 *
 * TEST INFRASTRUCTURE: used only by tests/ and bench.py's CPU legs.
 *
 * The reference answers "whom did object p meet" by locating p's keys in a
 * contact-tracing block (id_search_in_CTB / id_search_in_disk,
 * tracing/workbench.cpp:397-444): the object's sid selects its CTF (or the
 * oversize buffer, sid 1), CTF::binary_search finds its first key and the
 * walk of CTF::search_SSTable / oversize_buffer::search_buffer
 * (tracing/step_merge.cpp:67-115, 501-568) visits its keys; the targets of
 * hop k seed hop k+1 (search_multi_pid, tracing/process.cpp:476-495).  A key
 * (pid, target, duration, end) is a meeting [end - duration, end]; a time
 * window [t_start, t_end) keeps keys with start < t_end && t_start < end, the
 * predicate time_query was written for (util/query_context.h:95-104; the
 * reference itself runs with abandon = true, i.e. no window).
 *
 * Here the store's keys are given as edges (pid, target, start, end), one per
 * key.  Result: the objects first reached at each hop, in increasing id order,
 * seeds excluded.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "glint_oracle.h"

static int cmp_u32(const void *a, const void *b) {
    const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}

uint64_t go_query_bfs(const go_edge *edges, uint64_t n_edges, uint32_t num_objects, const uint32_t *seeds,
                      uint32_t n_seeds, uint32_t t_start, uint32_t t_end, uint32_t hops, uint32_t *out,
                      uint64_t cap, uint64_t *hop_end) {
    const uint32_t N = num_objects;
    /* CSR by pid */
    uint64_t *off = (uint64_t *)calloc((size_t)N + 1, sizeof(uint64_t));
    for (uint64_t e = 0; e < n_edges; ++e)
        if (edges[e].pid < N) off[edges[e].pid + 1]++;
    for (uint32_t i = 0; i < N; ++i) off[i + 1] += off[i];
    uint64_t *cur = (uint64_t *)malloc(sizeof(uint64_t) * (N ? N : 1));
    memcpy(cur, off, sizeof(uint64_t) * N);
    uint64_t *adj = (uint64_t *)malloc(sizeof(uint64_t) * (n_edges ? n_edges : 1));
    for (uint64_t e = 0; e < n_edges; ++e)
        if (edges[e].pid < N) adj[cur[edges[e].pid]++] = e;
    uint8_t *seen = (uint8_t *)calloc(N ? N : 1, 1);
    uint32_t *front = (uint32_t *)malloc(sizeof(uint32_t) * (N ? N : 1));
    uint32_t *next = (uint32_t *)malloc(sizeof(uint32_t) * (N ? N : 1));
    uint64_t nf = 0, total = 0;
    for (uint32_t i = 0; i < n_seeds; ++i)
        if (seeds[i] < N && !seen[seeds[i]]) {
            seen[seeds[i]] = 1;
            front[nf++] = seeds[i];
        }
    const int window = !(t_start == 0 && t_end == 0);
    for (uint32_t h = 0; h < hops; ++h) {
        uint64_t nn = 0;
        for (uint64_t f = 0; f < nf; ++f) {
            const uint32_t p = front[f];
            for (uint64_t k = off[p]; k < off[p + 1]; ++k) {
                const go_edge *e = &edges[adj[k]];
                if (window && !(e->start < t_end && t_start < e->end)) continue;
                if (e->target >= N || seen[e->target]) continue;
                seen[e->target] = 1;
                next[nn++] = e->target;
            }
        }
        qsort(next, nn, sizeof(uint32_t), cmp_u32);
        for (uint64_t i = 0; i < nn; ++i) {
            if (total + i < cap) out[total + i] = next[i];
        }
        total += nn;
        if (hop_end) hop_end[h] = total;
        uint32_t *t = front;
        front = next;
        next = t;
        nf = nn;
    }
    free(off); free(cur); free(adj); free(seen); free(front); free(next);
    return total;
}
