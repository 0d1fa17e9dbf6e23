// ov_frames.cu - frame files in the reference's text format (host code).
//
//  ov_write_frame   save_tangle / save_point / write_vector (utils.c:68-183)
//  ov_frame_slots   the slot count and empty-slot bookkeeping load_tangle
//                   leaves (utils.c:92-130, 185-199, with expand_tangle)
//  ov_read_frame    load_tangle into a caller tangle of that many slots
//                   (its next_empty / total_empty on entry are those of
//                   the tangle before the load)
//  ov_save_frame    a context's tangle (or ensemble member) to a frame file
//
// A frame line: loop index, position, velocity, tangent, normal (each three
// numbers in %.15g), then slot id, reverse, forward, status, pin wall.  The
// writer walks loops as save_tangle does, including its two tests that treat
// slot 0 as "no node" (utils.c:159, 166: `curr > 0`), so the files it writes
// are those of the reference; 17 significant digits can be asked for to
// make the file exact.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "ov_internal.cuh"

namespace {

void write_vec(FILE *f, const char *fmt3, const ov_vec3 &v) { fprintf(f, fmt3, v.p[0], v.p[1], v.p[2]); }

void write_point(FILE *f, const char *fmt3, int loop, const ov_tangle_state *t, int i)
{
    fprintf(f, "%d\t", loop);
    write_vec(f, fmt3, t->vnodes[i]);
    fprintf(f, "\t");
    write_vec(f, fmt3, t->vels[i]);
    fprintf(f, "\t");
    write_vec(f, fmt3, t->tangents[i]);
    fprintf(f, "\t");
    write_vec(f, fmt3, t->normals[i]);
    fprintf(f, "\t%d\t%d\t%d\t%d\t%d\n", i, t->connections[i].reverse, t->connections[i].forward, t->status[i].status,
            t->status[i].pin_wall);
}

struct FrameLine {
    int id;
    double v[12];
    int rev, fwd, status, pin;
};

// every line load_point would read (it stops at the first one fscanf cannot
// match completely)
int parse_frame(const char *path, std::vector<FrameLine> &out)
{
    FILE *f = fopen(path, "r");
    if (!f) return OV_ERR_ARG;
    out.clear();
    for (;;) {
        FrameLine L;
        int loop;
        int got = fscanf(f, "%d %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %lg %d %d %d %d %d", &loop, &L.v[0],
                         &L.v[1], &L.v[2], &L.v[3], &L.v[4], &L.v[5], &L.v[6], &L.v[7], &L.v[8], &L.v[9], &L.v[10],
                         &L.v[11], &L.id, &L.rev, &L.fwd, &L.status, &L.pin);
        if (got != 18) break;
        if (L.id < 0) { fclose(f); return OV_ERR_ARG; }
        out.push_back(L);
    }
    fclose(f);
    return OV_OK;
}

// The slot count, next_empty and total_empty after load_tangle into a
// tangle of n0 slots whose bookkeeping was (next_empty0, total_empty0)
// (create_tangle leaves 0 and n0): statuses reset for the n0 slots, then
// each line grows the tangle by doubling while its id does not fit
// (expand_tangle, tangle.c:68-101, which also runs get_next_empty_node on
// the statuses loaded so far).  Without growth the bookkeeping is left as
// it was, as load_point leaves it.
struct LoadBook {
    int n, next_empty, total_empty;
};

LoadBook simulate_load(const std::vector<FrameLine> &lines, int n0, int next_empty0, int total_empty0)
{
    LoadBook b{n0, next_empty0, total_empty0};
    std::vector<int> st(n0 > 0 ? n0 : 0, OV_EMPTY);
    auto search = [&]() -> int {   // search_next_empty_node (tangle.c:201-234)
        const int N = b.n;
        if (b.next_empty > 0 && b.next_empty < N && st[b.next_empty] == OV_EMPTY) {
            int id = b.next_empty;
            b.next_empty = (id + 1 < N && st[id + 1] == OV_EMPTY) ? id + 1 : -1;
            return id;
        }
        for (int k = 0; k < N; ++k)
            if (st[k] == OV_EMPTY) {
                b.next_empty = (k + 1 < N && st[k + 1] == OV_EMPTY) ? k + 1 : -1;
                return k;
            }
        return -1;
    };
    for (const FrameLine &L : lines) {
        while (L.id > b.n - 1) {
            const int old = b.n, n = 2 * b.n > 0 ? 2 * b.n : 1;
            st.resize(n, OV_EMPTY);
            b.n = n;
            b.total_empty += n - old;
            // get_next_empty_node: the tangle has free slots here, so no further growth
            int id = search();
            b.next_empty = id;
        }
        st[L.id] = L.status;
    }
    return b;
}

}  // namespace

extern "C" {

int ov_write_frame(const ov_tangle_state *t, const char *path, int digits)
{
    if (!t || !path || t->N < 0 || (digits != 15 && digits != 17)) return OV_ERR_ARG;
    if (t->N > 0 && (!t->vnodes || !t->vels || !t->tangents || !t->normals || !t->connections || !t->status))
        return OV_ERR_ARG;
    FILE *f = fopen(path, "w");
    if (!f) return OV_ERR_ARG;
    const char *fmt3 = digits == 17 ? "%.17g\t%.17g\t%.17g" : "%.15g\t%.15g\t%.15g";
    const int N = t->N;
    std::vector<char> visited(N > 0 ? N : 1, 0);
    int loop = 0;
    auto fwd = [&](int i) { return t->connections[i].forward; };
    auto rev = [&](int i) { return t->connections[i].reverse; };
    int status = OV_OK;
    for (int k = 0; k < N && status == OV_OK; ++k) {
        if (visited[k]) continue;
        if (t->status[k].status == OV_EMPTY) {
            visited[k] = 1;
            continue;
        }
        const int first = k;
        int curr = k;
        for (int guard = 0; fwd(curr) != first; ++guard) {
            if (guard > N) { status = OV_ERR_TOPOLOGY; break; }
            write_point(f, fmt3, loop, t, curr);
            visited[curr] = 1;
            curr = fwd(curr);
            if (curr < 0) {
                // an open line: the part behind the starting node, walking backwards
                curr = rev(first);
                for (int g2 = 0; curr > 0 && rev(curr) > 0; ++g2) {
                    if (g2 > N) { status = OV_ERR_TOPOLOGY; break; }
                    write_point(f, fmt3, loop, t, curr);
                    visited[curr] = 1;
                    curr = rev(curr);
                }
                break;
            }
            if (curr >= N) { status = OV_ERR_TOPOLOGY; break; }
        }
        if (status == OV_OK && curr > 0) {
            write_point(f, fmt3, loop, t, curr);
            visited[curr] = 1;
        }
        ++loop;
    }
    fclose(f);
    return status;
}

int ov_frame_slots(const char *path, int n0, int *n_slots, int *next_empty, int *total_empty)
{
    if (!path || n0 < 1) return OV_ERR_ARG;
    std::vector<FrameLine> lines;
    int r = parse_frame(path, lines);
    if (r) return r;
    LoadBook b = simulate_load(lines, n0, 0, n0);
    if (n_slots) *n_slots = b.n;
    if (next_empty) *next_empty = b.next_empty;
    if (total_empty) *total_empty = b.total_empty;
    return OV_OK;
}

int ov_read_frame(const char *path, int n0, ov_tangle_state *t)
{
    if (!path || !t || n0 < 1 || t->N < 0) return OV_ERR_ARG;
    std::vector<FrameLine> lines;
    int r = parse_frame(path, lines);
    if (r) return r;
    LoadBook b = simulate_load(lines, n0, t->next_empty, t->total_empty);
    if (t->N < b.n) return OV_ERR_ARG;   // size the tangle with ov_frame_slots first
    if (t->N > 0 && (!t->vnodes || !t->vels || !t->tangents || !t->normals || !t->connections || !t->status))
        return OV_ERR_ARG;
    for (int i = 0; i < t->N; ++i) {
        t->connections[i].forward = t->connections[i].reverse = -1;
        t->status[i].status = OV_EMPTY;
        t->status[i].pin_wall = OV_NOT_A_FACE;
    }
    for (const FrameLine &L : lines) {
        const int i = L.id;
        for (int a = 0; a < 3; ++a) {
            t->vnodes[i].p[a] = L.v[a];
            t->vels[i].p[a] = L.v[3 + a];
            t->tangents[i].p[a] = L.v[6 + a];
            t->normals[i].p[a] = L.v[9 + a];
        }
        t->connections[i].reverse = L.rev;
        t->connections[i].forward = L.fwd;
        t->status[i].status = L.status;
        t->status[i].pin_wall = L.pin;
    }
    t->next_empty = b.next_empty;
    t->total_empty = b.total_empty;
    return OV_OK;
}

int ov_save_frame(ov_ctx *c, int member, const char *path, int digits)
{
    if (!c || !path || member < 0 || member >= (int)c->mem.size()) return OV_ERR_ARG;
    const int n = c->mem[member].n;
    std::vector<ov_vec3> pos(n > 0 ? n : 1), vel(pos.size()), vs(pos.size()), tg(pos.size()), nm(pos.size());
    std::vector<ov_neighbour> conn(pos.size());
    std::vector<ov_node_status> st(pos.size());
    std::vector<int> rc(pos.size(), 0);
    ov_tangle_state t;
    memset(&t, 0, sizeof t);
    t.vnodes = pos.data(); t.vels = vel.data(); t.vs = vs.data(); t.tangents = tg.data(); t.normals = nm.data();
    t.recalculate = rc.data(); t.connections = conn.data(); t.status = st.data();
    t.N = n;
    int r = ov_download_member(c, member, &t, OV_F_ALL);
    if (r) return r;
    return ov_write_frame(&t, path, digits);
}

}  // extern "C"
