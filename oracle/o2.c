/*
 * oracle/o2.c -- TEST INFRASTRUCTURE ONLY (CPU baseline and distributional checker; never
 * linked into the product).
 *
 * O2: the reference's own data flow for the single-engine tick (thoughtworks/epirust,
 * engine/src/allocation_map.rs:67-134), restated in C with the rules of o_rules.h:
 *   - agents live in an FNV-1a-hashed open-addressing map keyed by their cell (the
 *     FnvHashMap<Point, Citizen> of allocation_map.rs:44-49), current and upcoming;
 *   - the map phase runs on a pool of threads over the current map in slot order and
 *     collects the updates in that order (rayon's par_iter().map().collect(), 82-92);
 *   - one thread then resolves conflicts in that order, first come first served, losers
 *     going back to their old cell (93-102), counts every agent, and swaps the maps (127-134).
 * Each agent-hour draws from Philox with a key different from O1's, so O2 trajectories are
 * independent samples of the same model; O2 and O1 agree in distribution, not bit for bit.
 */
#define _POSIX_C_SOURCE 200809L
#include <pthread.h>
#include <stdlib.h>

#include "o_common.h"

#define EMPTY_KEY 0xFFFFFFFFu

typedef struct { uint32_t key; citizen c; } slot;
typedef struct { slot* slots; uint32_t mask; uint32_t count; } hmap;

/* FNV-1a 64 over the 8 bytes of Point { x: i32, y: i32 } (little endian) */
static inline uint64_t fnv_point(uint32_t key) {
    uint32_t x = key & 0xFFFFu, y = key >> 16;
    uint64_t h = 0xcbf29ce484222325ull;
    uint8_t b[8] = {(uint8_t)x, (uint8_t)(x >> 8), 0, 0, (uint8_t)y, (uint8_t)(y >> 8), 0, 0};
    for (int i = 0; i < 8; ++i) { h ^= b[i]; h *= 0x100000001b3ull; }
    return h;
}
static inline uint32_t pkey(pt p) { return (uint32_t)p.x | ((uint32_t)p.y << 16); }
static inline pt kpt(uint32_t k) { pt p; p.x = (int32_t)(k & 0xFFFFu); p.y = (int32_t)(k >> 16); return p; }

static int64_t hfind(const hmap* m, uint32_t key) {
    uint32_t i = (uint32_t)fnv_point(key) & m->mask;
    while (m->slots[i].key != EMPTY_KEY) {
        if (m->slots[i].key == key) return i;
        i = (i + 1) & m->mask;
    }
    return -1;
}
/* entry(key).or_insert(c): returns the slot holding key (inserting c if absent) */
static uint32_t hentry(hmap* m, uint32_t key, const citizen* c) {
    uint32_t i = (uint32_t)fnv_point(key) & m->mask;
    while (m->slots[i].key != EMPTY_KEY) {
        if (m->slots[i].key == key) return i;
        i = (i + 1) & m->mask;
    }
    m->slots[i].key = key;
    m->slots[i].c = *c;
    m->count++;
    return i;
}
static void hinsert(hmap* m, uint32_t key, const citizen* c) {
    uint32_t i = hentry(m, key, c);
    m->slots[i].c = *c;
}
static void hclear(hmap* m) {
    for (uint32_t i = 0; i <= m->mask; ++i) m->slots[i].key = EMPTY_KEY;
    m->count = 0;
}

#define SNAP_T hmap
static inline int snap_vacant(const hmap* m, pt p) { return hfind(m, pkey(p)) < 0; }
static inline const citizen* snap_get(const hmap* m, pt p) {
    int64_t i = hfind(m, pkey(p));
    return i < 0 ? NULL : &m->slots[i].c;
}
#include "o_rules.h"

typedef struct { uint32_t old_key; pt nc; citizen c; } update;

typedef struct o2_sim o2_sim;
typedef struct { o2_sim* s; int tid; } worker_arg;

struct o2_sim {
    o_world w;
    uint32_t n;
    hmap cur, nxt;
    update* updates;
    uint32_t* chunk_count;
    int threads;
    pthread_t* tids;
    worker_arg* args;
    pthread_barrier_t start, done;
    int quit;
    uint32_t hour;
    o_iv_state iv;
};

static void map_chunk(o2_sim* s, int t, int write) {
    uint32_t cap = s->cur.mask + 1;
    uint32_t lo = (uint32_t)((uint64_t)cap * t / s->threads), hi = (uint32_t)((uint64_t)cap * (t + 1) / s->threads);
    if (!write) {
        uint32_t k = 0;
        for (uint32_t i = lo; i < hi; ++i) k += s->cur.slots[i].key != EMPTY_KEY;
        s->chunk_count[t] = k;
        return;
    }
    uint32_t out = 0;
    for (int j = 0; j < t; ++j) out += s->chunk_count[j];
    for (uint32_t i = lo; i < hi; ++i) {
        const slot* sl = &s->cur.slots[i];
        if (sl->key == EMPTY_KEY) continue;
        update* u = &s->updates[out++];
        draws d;
        draws_init(&d, &s->w, sl->c.id, s->hour);
        u->old_key = sl->key;
        u->c = sl->c;
        u->nc = routine(&s->w, &s->cur, &u->c, kpt(sl->key), s->hour, &d);
    }
}

static void* worker(void* arg) {
    worker_arg* a = (worker_arg*)arg;
    o2_sim* s = a->s;
    for (;;) {
        pthread_barrier_wait(&s->start);
        if (s->quit) break;
        map_chunk(s, a->tid, 0);
        pthread_barrier_wait(&s->done);
        pthread_barrier_wait(&s->start);
        map_chunk(s, a->tid, 1);
        pthread_barrier_wait(&s->done);
    }
    return NULL;
}

static void parallel_map(o2_sim* s) {
    for (int pass = 0; pass < 2; ++pass) {
        pthread_barrier_wait(&s->start);
        map_chunk(s, 0, pass);
        pthread_barrier_wait(&s->done);
    }
}

/* CitizenLocationMap::simulate with the reference order semantics. */
int o2_simulate(o2_sim* s, uint32_t hour, uint32_t out_counts[6]) {
    uint32_t cnt[6] = {0, 0, 0, 0, 0, 0};
    s->hour = hour;
    parallel_map(s);
    for (uint32_t k = 0; k < s->n; ++k) {
        const update* u = &s->updates[k];
        uint32_t i = hentry(&s->nxt, pkey(u->nc), &u->c);
        if (s->nxt.slots[i].c.id != u->c.id) hinsert(&s->nxt, u->old_key, &u->c);
        count_agent(cnt, &u->c);
    }
    hclear(&s->cur);
    hmap t = s->cur; s->cur = s->nxt; s->nxt = t;
    uint32_t total = 0;
    for (int k = 0; k < 6; ++k) total += cnt[k];
    if (out_counts) memcpy(out_counts, cnt, sizeof cnt);
    return total == s->n && s->cur.count == s->n ? EPI_OK : EPI_ERR_INVARIANT;
}

uint32_t o2_process_interventions(o2_sim* s, uint32_t hour, const uint32_t c[6]) {
    o_iv_actions a = o_decide_interventions(&s->w, &s->iv, hour, c);
    for (uint32_t i = 0; i <= s->cur.mask; ++i) {
        slot* sl = &s->cur.slots[i];
        if (sl->key == EMPTY_KEY) continue;
        citizen* r = &sl->c;
        if (a.vaccinate && r->state == EPI_S) {
            uint32_t u[4];
            draw4(&s->w, r->id, hour, 3u, u);
            if (bern(u[0], a.percent)) r->vaccinated = 1;
        }
        if (a.lock && r->ws != EPI_WS_ESSENTIAL) r->isolated = 1;
        if (a.unlock && r->isolated) r->isolated = 0;
    }
    if (a.grow) o_increase_hospital_size(&s->w);
    return a.applied;
}

int o2_run(o2_sim* s, uint32_t first_hour, uint32_t last_hour_excl, uint32_t* rows, uint32_t* n_rows,
           int with_interventions, int with_stop) {
    uint32_t k = 0;
    for (uint32_t hour = first_hour; hour < last_hour_excl; ++hour) {
        uint32_t c[6];
        int st = o2_simulate(s, hour, c);
        if (st) { *n_rows = k; return st; }
        if (rows) { rows[7 * k] = hour; memcpy(&rows[7 * k + 1], c, sizeof c); }
        ++k;
        if (with_interventions) o2_process_interventions(s, hour, c);
        if (with_stop && c[1] == 0 && c[2] == 0 && c[3] == 0) break;
    }
    *n_rows = k;
    return EPI_OK;
}

void o_import_citizen(const epi_agent_record* r, uint32_t id, citizen* c, pt* pos);
void o_export_citizen(const citizen* c, pt pos, epi_agent_record* r);

void o2_free(o2_sim* s) {
    if (!s) return;
    if (s->tids) {
        s->quit = 1;
        pthread_barrier_wait(&s->start);
        for (int t = 1; t < s->threads; ++t) pthread_join(s->tids[t], NULL);
        pthread_barrier_destroy(&s->start);
        pthread_barrier_destroy(&s->done);
    }
    free(s->cur.slots); free(s->nxt.slots); free(s->updates); free(s->chunk_count); free(s->tids); free(s->args);
    free(s);
}

/* Build from records; threads = size of the map-phase pool (the reference's -t). */
o2_sim* o2_create_from_records(const epi_params* p, const epi_agent_record* recs, uint32_t n, int threads, int* status) {
    o2_sim* s = (o2_sim*)calloc(1, sizeof(o2_sim));
    epi_params q = *p;
    q.number_of_agents = n;
    q.seed = p->seed ^ 0x9E3779B97F4A7C15ull;  /* a stream independent of O1's */
    *status = o_world_init(&s->w, &q);
    if (*status) return s;
    o_resize_hospital(&s->w, (int32_t)n, 0.002, p->hospital_beds_percentage);
    s->n = n;
    uint32_t cap = 16;
    while (cap < 2u * n) cap <<= 1;
    s->cur.slots = (slot*)malloc((size_t)cap * sizeof(slot));
    s->nxt.slots = (slot*)malloc((size_t)cap * sizeof(slot));
    s->updates = (update*)malloc((size_t)(n ? n : 1) * sizeof(update));
    s->threads = threads < 1 ? 1 : threads;
    s->chunk_count = (uint32_t*)calloc((size_t)s->threads, sizeof(uint32_t));
    if (!s->cur.slots || !s->nxt.slots || !s->updates || !s->chunk_count) { *status = EPI_ERR_CAPACITY; return s; }
    s->cur.mask = s->nxt.mask = cap - 1;
    hclear(&s->cur);
    hclear(&s->nxt);
    for (uint32_t i = 0; i < n; ++i) {
        citizen c;
        pt q0;
        o_import_citizen(&recs[i], i, &c, &q0);
        if (q0.x < 0 || q0.y < 0 || q0.x > s->w.G || q0.y > s->w.G || hfind(&s->cur, pkey(q0)) >= 0) {
            *status = EPI_ERR_ARG;
            return s;
        }
        hentry(&s->cur, pkey(q0), &c);
    }
    pthread_barrier_init(&s->start, NULL, (unsigned)s->threads);
    pthread_barrier_init(&s->done, NULL, (unsigned)s->threads);
    s->tids = (pthread_t*)calloc((size_t)s->threads, sizeof(pthread_t));
    s->args = (worker_arg*)calloc((size_t)s->threads, sizeof(worker_arg));
    for (int t = 1; t < s->threads; ++t) {
        s->args[t].s = s;
        s->args[t].tid = t;
        pthread_create(&s->tids[t], NULL, worker, &s->args[t]);
    }
    *status = EPI_OK;
    return s;
}

/* Agents back in creation order. */
void o2_export(const o2_sim* s, epi_agent_record* out) {
    for (uint32_t i = 0; i <= s->cur.mask; ++i) {
        const slot* sl = &s->cur.slots[i];
        if (sl->key == EMPTY_KEY) continue;
        o_export_citizen(&sl->c, kpt(sl->key), &out[sl->c.id]);
    }
}
