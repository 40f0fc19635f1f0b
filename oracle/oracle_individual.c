/*
 * oracle_individual.c -- CPU restatement of SimInf's cleaning of
 * individual-based event data (src/misc/SimInf_individual_events.c).
 * TEST INFRASTRUCTURE: only the test suite and the CPU-baseline leg of the
 * benchmark load it; the product never links it.
 *
 * Input: events sorted by (id, time, event, node, dest) with duplicates
 * removed, as R/SimInf_individual_events.R:397-410 hands them to the C
 * code; event 0 (exit), 1 (enter) or 3 (external transfer); dest is R's
 * NA (INT_MIN) except for external transfers.  Output: keep[i] = 1 for the
 * events on each individual's longest consistent path, else 0.
 *
 * Per individual (SimInf_find_longest_path, :50-147): when any event is an
 * enter, a path must begin with an enter; when any is an exit, a kept path
 * must end with an exit.  A path continues from the node an event leaves
 * the individual in (node of an enter, dest of a transfer) to a later event
 * that starts there, is an exit or a transfer, and does not lead back to
 * that node.  Every admissible first event roots a depth-first search whose
 * branches are tried in array order; a path replaces the best one only when
 * strictly longer, so the first longest path found wins ties.  A lone first
 * event is kept when nothing better exists: an enter or a transfer if no
 * exit is present, an exit if one is.
 *
 * The search order, the tie rule and the stopping rules (a root stops as
 * soon as its path can no longer grow, :94) are kept exactly, since they
 * decide which of several equally long paths survives.
 */
#include <limits.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { IE_EXIT = 0, IE_ENTER = 1, IE_EXTERNAL_TRANSFER = 3 };

/* The events of one individual: [0, n) of each column. */
typedef struct {
    const int *event, *time, *node, *dest;
    long long n;
} ie_group;

/* May event j follow event i on a path? */
static int ie_follows(const ie_group *g, long long i, long long j)
{
    const int at = g->event[i] == IE_ENTER ? g->node[i] : g->dest[i];
    return g->time[j] > g->time[i] && g->node[j] == at && g->dest[j] != at &&
           (g->event[j] == IE_EXIT || g->event[j] == IE_EXTERNAL_TRANSFER);
}

/* The longest path of one individual; path is scratch of n ints (one-based
 * event positions, 0 = empty), keep is zero on entry. */
static void ie_longest_path(const ie_group *g, int *path, int *keep)
{
    const long long n = g->n;
    int any_enter = 0, any_exit = 0;
    for (long long i = 0; i < n; i++) {
        any_enter |= g->event[i] == IE_ENTER;
        any_exit |= g->event[i] == IE_EXIT;
    }

    long long best = 0;
    for (long long root = 0; root < n; root++) {
        const int er = g->event[root];
        if (any_enter && er != IE_ENTER)
            continue;
        if (best == 0 && (any_exit ? er == IE_EXIT
                                   : (er == IE_ENTER || er == IE_EXTERNAL_TRANSFER))) {
            best = 1;
            keep[root] = 1;
        }

        memset(path, 0, (size_t) n * sizeof(int));
        path[0] = (int) (root + 1);
        const long long room = n - root;     /* no path from this root is longer */
        long long depth = 1;
        while (depth > 0 && depth < room && best < room) {
            const long long prev = path[depth - 1] - 1;
            /* resume after the branch tried last at this depth, if any */
            long long j = path[depth] > 0 ? path[depth] : prev + 1;
            path[depth] = 0;
            for (; j < n; j++) {
                if (!ie_follows(g, prev, j))
                    continue;
                path[depth] = (int) (j + 1);
                const int ends_open = any_exit && g->event[j] == IE_EXTERNAL_TRANSFER;
                if (!ends_open && depth + 1 > best) {
                    best = depth + 1;
                    memset(keep, 0, (size_t) n * sizeof(int));
                    for (long long k = 0; k < best; k++)
                        keep[path[k] - 1] = 1;
                }
                break;
            }
            if (path[depth] == 0) {
                depth--;                      /* no branch left: back up */
            } else if (g->event[path[depth] - 1] == IE_EXIT) {
                path[depth] = 0;              /* an exit ends the path */
                depth--;
            } else {
                depth++;
            }
        }
    }
}

/* Returns -1 when every event type is valid, else the zero-based index of
 * the first invalid one (the reference's "'event[i]' is invalid.", :210). */
long long oracle_individual_events_check(long long len, const int *event)
{
    for (long long i = 0; i < len; i++)
        if (event[i] != IE_EXIT && event[i] != IE_ENTER && event[i] != IE_EXTERNAL_TRANSFER)
            return i;
    return -1;
}

/* keep[0 .. len) for sorted, de-duplicated events; individuals (runs of
 * equal id) are searched in parallel over `threads` OpenMP threads, as the
 * reference spawns one task per individual (:229-244).  Returns 0, or -1
 * with *bad set for an invalid event type (keep then all zero). */
int oracle_individual_events(long long len, const int *id, const int *event, const int *time,
                             const int *node, const int *dest, int *keep, int threads,
                             long long *bad)
{
    memset(keep, 0, (size_t) (len > 0 ? len : 0) * sizeof(int));
    *bad = oracle_individual_events_check(len, event);
    if (*bad >= 0)
        return -1;
    if (len <= 0)
        return 0;
    /* group starts, then the groups in parallel */
    long long ngroups = 0;
    long long *start = (long long *) malloc((size_t) (len + 1) * sizeof(long long));
    int *path = (int *) malloc((size_t) len * sizeof(int));
    if (!start || !path) {
        free(start);
        free(path);
        return -2;
    }
    for (long long i = 0; i < len; i++)
        if (i == 0 || id[i] != id[i - 1])
            start[ngroups++] = i;
    start[ngroups] = len;
    if (threads < 1)
        threads = 1;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
    for (long long k = 0; k < ngroups; k++) {
        const long long b = start[k];
        const ie_group g = {event + b, time + b, node + b, dest + b, start[k + 1] - b};
        ie_longest_path(&g, path + b, keep + b);
    }
    free(start);
    free(path);
    return 0;
}
