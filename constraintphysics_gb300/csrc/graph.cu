// graph.cu — persistent contact graph and islands on the device.
//
// Contact persistence (PhysicsEngine::addContact, PhysicsEngine.cpp:1062-1111;
// expiry :1434-1446): the edge list of the previous step (sorted by the pair
// key) loses its expired contacts and empty edges, and is merged with this
// step's manifolds.  Both lists are sorted, so every element finds its output
// position by a binary search in the other list plus an exclusive scan; no sort
// is needed.  Within an edge, surviving contacts keep their order, manifold
// points update the first contact with the same MagicID or are appended.
//
// Islands and row order (PhysicsEngine::sleepOrSolveIslands / bfsVisitAll,
// PhysicsEngine.cpp:1260-1283, 1536-1613): one block per world builds the
// adjacency of dynamic bodies sorted by the other body id
// (ConstraintGraphNode::insertNewEdge, :1984-1995), then a depth-first search
// (LIFO stack) starts from every unvisited dynamic body in constraint-graph
// node-map iteration order (supplied by the host) and emits each live contact
// of each edge to a not-yet-visited neighbour, in per-edge order.  That is the
// reference's exact row order.  Worlds above kTileWorld bodies search their
// connected components in parallel (islands_big), with the same result.
#include "kernels.cuh"
#include "devmath.cuh"

namespace cpgpu {

namespace {

constexpr int kMaxEdgeContacts = 64;

__device__ __forceinline__ int lower_bound_u64(const uint64_t* keys, int n, uint64_t k) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (keys[m] < k) lo = m + 1; else hi = m;
    }
    return lo;
}
__device__ __forceinline__ uint64_t pair_key(const Dev& d, int p) {
    return ((uint64_t)(uint32_t)d.pair_a[p] << 32) | (uint32_t)d.pair_b[p];
}
__device__ __forceinline__ int lower_bound_pairs(const Dev& d, int n, uint64_t k) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (pair_key(d, m) < k) lo = m + 1; else hi = m;
    }
    return lo;
}

__global__ void k_surv(Dev d) {
    const int n = *d.n_edges_old;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        int s = d.e_old.cstart[e], c = d.e_old.ccount[e], alive = 0;
        for (int k = s; k < s + c; k++) alive += !cs_dead(d.c_old.state[k]);
        d.surv[e] = alive > 0;
    }
}

__global__ void k_pair_match(Dev d) {
    const int np = *d.n_pairs, ne = *d.n_edges_old;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        bool hasm = d.mf_n[p].w > 0.f;
        uint64_t key = pair_key(d, p);
        int e = lower_bound_u64(d.e_old.key, ne, key);
        bool matched = e < ne && d.e_old.key[e] == key && d.surv[e];
        d.pair_edge[p] = matched ? e : -1;
        d.unm[p] = hasm && !matched;
    }
}

// cnt[0] = surviving old edges, cnt[1] = unmatched manifolds (both from scans)
__global__ void k_place(Dev d, const int* cnt) {
    const int ne = *d.n_edges_old, np = *d.n_pairs;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (int e = tid; e < ne; e += stride) {
        if (!d.surv[e]) continue;
        uint64_t key = d.e_old.key[e];
        int r = lower_bound_pairs(d, np, key);
        int ub = (r < np) ? d.unm_scan[r] : cnt[1];
        int pos = d.surv_scan[e] + ub;
        if (pos < d.cap_edges) {
            d.e_new.key[pos] = key;
            d.edge_src[pos] = e;
            d.edge_pair[pos] = (r < np && pair_key(d, r) == key && d.mf_n[r].w > 0.f) ? r : -1;
        }
    }
    for (int p = tid; p < np; p += stride) {
        if (!d.unm[p]) continue;
        uint64_t key = pair_key(d, p);
        int r = lower_bound_u64(d.e_old.key, ne, key);
        int sb = (r < ne) ? d.surv_scan[r] : cnt[0];
        int pos = d.unm_scan[p] + sb;
        if (pos < d.cap_edges) {
            d.e_new.key[pos] = key;
            d.edge_src[pos] = -1;
            d.edge_pair[pos] = p;
        }
    }
}

__global__ void k_edge_total(Dev d, const int* cnt) {
    int n = cnt[0] + cnt[1];
    if (n > d.cap_edges) { atomicOr(d.status, ST_EDGE_OVERFLOW); n = d.cap_edges; }
    *d.n_edges_new = n;
}

__global__ void k_contact_total(Dev d) {
    if (*d.n_contacts_new > d.cap_contacts) { atomicOr(d.status, ST_CONTACT_OVERFLOW); *d.n_contacts_new = d.cap_contacts; }
}

// per new edge: surviving old contacts (in order), then this step's manifold
// points matched by MagicID or appended
__global__ void k_contacts(Dev d, int write) {
    const int ne = *d.n_edges_new;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        int ids[kMaxEdgeContacts];
        signed char upd[kMaxEdgeContacts];
        uint64_t mags[kMaxEdgeContacts];
        int tris[kMaxEdgeContacts];
        int n = 0;
        const int src = d.edge_src[e], p = d.edge_pair[e];
        if (src >= 0) {
            int s = d.e_old.cstart[src], c = d.e_old.ccount[src];
            for (int k = s; k < s + c; k++) {
                if (cs_dead(d.c_old.state[k])) continue;
                if (n < kMaxEdgeContacts) { ids[n] = k; mags[n] = d.c_old.magic[k]; tris[n] = d.c_old.tri[k]; upd[n] = -1; n++; }
                else atomicOr(d.status, ST_CONTACT_OVERFLOW);
            }
        }
        // a mesh pair's points (each with its merged manifold's normal) are in
        // the mesh store; the MagicID's cID then carries the triangle id
        const int mofs = (p >= 0 && (d.has_mesh || d.has_union)) ? d.mf_ofs[p] : -1;
        int np = (p >= 0) ? d.mf_cnt[p] : 0;
        for (int k = 0; k < np; k++) {
            uint64_t m = mofs >= 0 ? d.mm_magic[mofs + k] : d.mf_magic[4 * p + k];
            int t = mofs >= 0 ? d.mm_tri[mofs + k] : 0;
            int j = 0;
            while (j < n && (mags[j] != m || tris[j] != t)) j++;
            if (j < n) upd[j] = (signed char)k;
            else if (n < kMaxEdgeContacts) { ids[n] = -1; mags[n] = m; tris[n] = t; upd[n] = (signed char)k; n++; }
            else atomicOr(d.status, ST_CONTACT_OVERFLOW);
        }
        if (!write) { d.edge_cnt[e] = n; continue; }
        const int base = d.e_new.cstart[e];
        if (base + n > d.cap_contacts) n = base < d.cap_contacts ? d.cap_contacts - base : 0;
        d.e_new.ccount[e] = n;
        const uint64_t key = d.e_new.key[e];
        const int b1 = (int)(key >> 32), b2 = (int)(key & 0xffffffffu);
        M33 i1 = quatRot(qconj(d.rot[b1])), i2 = quatRot(qconj(d.rot[b2]));
        f3 c1 = mk(d.pos[b1]), c2 = mk(d.pos[b2]);
        float4 m1 = d.material[b1], m2 = d.material[b2];
        float rest = fmaxf(m1.x, m2.x), kin = (m1.y + m2.y) / 2.0f, sta = (m1.z + m2.z) / 2.0f;
        const WorldParams& wp = d.wparams[d.world[b1]];
        const bool u1 = d.has_union && d.prim_start[b1] >= 0, u2 = d.has_union && d.prim_start[b2] >= 0;
        const bool with_mesh = reinterpret_cast<const HullHeader*>(d.shapes + d.shape[b1])->kind == SHAPE_MESH ||
                               reinterpret_cast<const HullHeader*>(d.shapes + d.shape[b2])->kind == SHAPE_MESH;
        for (int j = 0; j < n; j++) {
            if (u1 || u2) {
                // a body of several primitives: the touching primitives'
                // materials (each primitive carries its own)
                const int t = tris[j];
                float4 q1 = m1, q2 = m2;
                if (with_mesh) {
                    if (u1) q1 = d.prim_mat[d.prim_start[b1] + ((t >> 24) & 0xff)];
                    if (u2) q2 = d.prim_mat[d.prim_start[b2] + ((t >> 24) & 0xff)];
                } else {
                    if (u1) q1 = d.prim_mat[d.prim_start[b1] + ((t >> 8) & 0xff)];
                    if (u2) q2 = d.prim_mat[d.prim_start[b2] + (t & 0xff)];
                }
                rest = fmaxf(q1.x, q2.x); kin = (q1.y + q2.y) / 2.0f; sta = (q1.z + q2.z) / 2.0f;
            }
            int dst = base + j;
            const ContactStore& O = d.c_old;
            const ContactStore& N = d.c_new;
            float4 p1, p2, nn, imp, fu, fw;
            int st;
            if (ids[j] >= 0) {
                int o = ids[j];
                p1 = O.p1[o]; p2 = O.p2[o]; nn = O.n[o]; imp = O.imp[o]; fu = O.fu[o]; fw = O.fw[o]; st = O.state[o];
            } else {
                p2.w = rest;
                nn.w = kin;
                imp = make_float4(0.f, 0.f, 0.f, 0.f);
                fu = fw = make_float4(0.f, 0.f, 0.f, 0.f);
                st = cs_make(0, false, false, false);
            }
            if (upd[j] >= 0) {
                float4 pt = mofs >= 0 ? d.mm_pt[mofs + upd[j]] : d.mf_pt[4 * p + upd[j]];
                f3 pos = mk(pt);
                f3 nw = mk(mofs >= 0 ? d.mm_n[mofs + upd[j]] : d.mf_n[p]);
                f3 nl = mul(i1, nw), l1 = mul(i1, pos - c1), l2 = mul(i2, pos - c2);
                float fc = (ids[j] >= 0) ? (cs_static(st) ? sta : kin) : kin;
                p1 = make_float4(l1.x, l1.y, l1.z, pt.w);
                p2 = make_float4(l2.x, l2.y, l2.z, p2.w);
                nn = make_float4(nl.x, nl.y, nl.z, fc);
                st = cs_make(wp.contact_life, true, cs_static(st), false);
            }
            N.magic[dst] = mags[j];
            N.p1[dst] = p1; N.p2[dst] = p2; N.n[dst] = nn; N.imp[dst] = imp; N.fu[dst] = fu; N.fw[dst] = fw;
            N.state[dst] = st;
            N.edge[dst] = e;
            N.tri[dst] = tris[j];
        }
    }
}

// ---- islands: one block per world ---------------------------------------------------
// The world's graph (body flags, adjacency, DFS stack, live-contact counts) is
// built in dynamic shared memory when it fits the launch's budget: the serial
// DFS below is a chain of dependent loads, about 30 cycles each from shared
// memory instead of several hundred from L2.  A world that does not fit runs
// the same code over its slices of the global scratch arrays.  All indices
// here are world-local: body i - s, contact edge k - e0 (joint edges keep
// their global index, stored as -(k + 1)).
__device__ __forceinline__ long long islands_need(int nb, int ne_w, int nj) {
    const long long E = (long long)ne_w + nj;
    return 4LL * (5LL * nb + 4 * E + ne_w + 2 * E + nb) + nb;   // ints, then the body flags (bytes)
}

// ---- islands of large worlds: one DFS per connected component ----------------
// The reference's search starts from each unvisited dynamic body in map order
// and covers that body's component (dynamic bodies joined by edges; fixed and
// kinematic bodies end it), so each island is the component of its first body
// in map order, searched from there; its rows depend on nothing outside it.
// Components are found by a union-find over the adjacency, listed in the map
// order of their first bodies, searched once to count their rows, bodies and
// systems, and once more to write them at the prefix of those counts.  The
// result is the serial search's, position for position.

// exclusive prefix of one value per thread (blockDim.x == 256) with the
// block's total in *total; `ws` holds 8 ints
__device__ int block_excl(int v, int* ws, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += t; }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int y = lane < 8 ? ws[lane] : 0;
        for (int o = 1; o < 8; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, y, o); if (lane >= o) y += t; }
        if (lane < 8) ws[lane] = y;
    }
    __syncthreads();
    const int incl = x + (wid > 0 ? ws[wid - 1] : 0);
    *total = ws[7];
    __syncthreads();
    return incl - v;
}

__device__ __forceinline__ int uf_root(int* par, int x) {
    while (true) {
        const int p = atomicAdd(&par[x], 0);
        if (p == x) return x;
        const int g = atomicAdd(&par[p], 0);
        if (g != p) atomicCAS(&par[x], p, g);   // path halving
        x = p;
    }
}
__device__ void uf_link(int* par, int a, int b) {
    while (true) {
        a = uf_root(par, a);
        b = uf_root(par, b);
        if (a == b) return;
        if (a > b) { const int t = a; a = b; b = t; }
        if (atomicCAS(&par[b], b, a) == b) return;   // the larger root under the smaller
    }
}

struct IslandCtx {
    int w, s, e0, ready_steps;
    bool sleep_on, may_sleep, joints;
    const int *a_ofs, *a_cur, *adj, *live;
    const uint8_t* mov;
    int* vis;
};

// One component's search from `root` (the serial search's loop body).  COUNT:
// marks its bodies -2 and returns its rows, bodies, systems and whether all of
// them are ready to sleep; otherwise writes bodies at bc, rows at rc and
// systems at sc (or, for a component that falls asleep, puts it to sleep).
template <bool COUNT>
__device__ void island_search(const Dev& d, const IslandCtx& x, int root, int* stk, int cap, int rc, int bc, int sc,
                              bool sleeps, int comp_id, int* o_rows, int* o_bodies, int* o_sys, bool* o_ready,
                              bool* o_joint) {
    const int rs = rc, bs = bc, ss = sc;
    int sp = 0, nbod = 0, nsys = 0;
    bool all_ready = true, has_joint = false;
    stk[sp++] = root;
    while (sp > 0) {
        const int cur = stk[--sp];
        if (COUNT ? x.vis[cur] == -2 : x.vis[cur] >= 0) continue;
        if (COUNT) x.vis[cur] = -2;
        else {
            x.vis[cur] = bc - bs;
            if (sleeps) {
                const int g = cur + x.s;
                d.asleep[g] = 1;
                d.vel[g] = make_float4(0.f, 0.f, 0.f, 0.f);
                d.angv[g] = make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                d.isl_bodies[bc] = cur + x.s;
            }
            bc++;
        }
        nbod++;
        const int lo = x.a_ofs[cur], hi = x.a_cur[cur];
        const bool cur_asleep = x.sleep_on && d.asleep[cur + x.s];
        bool kinematic_contact = false;
        for (int j = lo; j < hi; j++) {
            const int o = x.adj[2 * j], k = x.adj[2 * j + 1];
            if (x.mov[o] == 2) kinematic_contact = true;
            if (COUNT ? x.vis[o] == -2 : x.vis[o] >= 0) continue;
            if (cur_asleep && (x.mov[o] == 1 || d.asleep[o + x.s])) {
                // no rows; the neighbour still joins the island
            } else if (k < 0) {
                const int je = -k - 1, sy = d.je.sys[je];
                if (sy >= 0) {
                    if (COUNT) {
                        if (d.sys_mark[sy] != comp_id) { d.sys_mark[sy] = comp_id; nsys++; }
                    } else if (!sleeps) {
                        bool seen = false;
                        for (int q = ss; q < sc; q++) seen |= d.isl_sys[q] == sy;
                        if (!seen) d.isl_sys[sc++] = sy;
                    }
                }
                for (int q = d.je.jstart[je]; q < d.je.jstart[je] + d.je.jcount[je]; q++) {
                    const int jj = d.je.jlist[q];
                    if (jk_conditional(d.jt.kind[jj]) && !d.jt.active[jj]) continue;
                    if (!COUNT && !sleeps) d.row_contact[rc] = -(jj + 1);
                    rc++;
                    has_joint = true;
                }
            } else {
                const int nl = x.live[k];
                if (nl > 0) {
                    if (!COUNT && !sleeps) d.edge_row[x.e0 + k] = rc;
                    rc += nl;
                }
            }
            if (x.mov[o] == 0) {
                if (sp < cap) stk[sp++] = o;
                else atomicOr(d.status, ST_STACK_OVERFLOW);
            }
        }
        if (x.may_sleep && (kinematic_contact || d.ready_cnt[cur + x.s] < x.ready_steps)) all_ready = false;
    }
    if (COUNT) {
        *o_rows = rc - rs;
        *o_bodies = nbod;
        *o_sys = nsys;
        *o_ready = all_ready;
        *o_joint = has_joint;
    }
}

// the component-parallel island pass of one large world (all threads of the block)
__device__ void islands_big(const Dev& d, const IslandCtx& x, int nb, int row0, int sys0, int* ws, int* sh_rows_end) {
    const int* map_g = d.map_order + x.s;   // map order, global body indices
    const int tid = threadIdx.x, nt = blockDim.x;
    int* C = d.comp + (size_t)kCompArrays * x.s;   // this world's scratch: kCompArrays slices of nb
    int* par = C;                 // union-find parent
    int* cmin = C + nb;           // per root: first map position of its component
    int* deg = C + 2 * nb;        // per root: its component's adjacency entries
    int* list = C + 3 * nb;       // components in map order of their first bodies (root body)
    int* stk_off = C + 4 * nb;    // per component: its stack slice
    int* n_rows = C + 5 * nb;
    int* n_bod = C + 6 * nb;
    int* n_sys = C + 7 * nb;
    int* kind = C + 8 * nb;       // 0 none, 1 island, 2 falls asleep
    int* o_rows = C + 9 * nb;
    int* o_bod = C + 10 * nb;
    int* o_sys = C + 11 * nb;
    __shared__ int sh_tot, sh_ncomp;
    for (int i = tid; i < nb; i += nt) { par[i] = i; cmin[i] = INT_MAX; deg[i] = 0; }
    if (x.joints)   // last step's component ids are no marks for this step
        for (int q = d.hs_world_start[x.w] + tid; q < d.hs_world_start[x.w + 1]; q += nt) d.sys_mark[q] = -1;
    __syncthreads();
    for (int i = tid; i < nb; i += nt) {
        if (x.mov[i] != 0) continue;
        for (int j = x.a_ofs[i]; j < x.a_cur[i]; j++) {
            const int o = x.adj[2 * j];
            if (x.mov[o] == 0 && o > i) uf_link(par, i, o);
        }
    }
    __syncthreads();
    for (int t = tid; t < nb; t += nt) {
        const int node = map_g[t] - x.s;
        if (x.mov[node] != 0) continue;
        const int r = uf_root(par, node);
        atomicMin(&cmin[r], t);
        atomicAdd(&deg[r], x.a_cur[node] - x.a_ofs[node]);
    }
    __syncthreads();
    // the components' roots listed in map order of their first bodies
    if (tid == 0) sh_ncomp = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += nt) {
        const int t = base + tid;
        int node = -1, flag = 0;
        if (t < nb) {
            node = map_g[t] - x.s;
            flag = x.mov[node] == 0 && cmin[uf_root(par, node)] == t;
        }
        int tot;
        const int pos = block_excl(flag, ws, &tot);
        const int k0 = sh_ncomp;
        if (flag) list[k0 + pos] = node;
        __syncthreads();
        if (tid == 0) sh_ncomp = k0 + tot;
        __syncthreads();
    }
    const int K = sh_ncomp;
    // stack slices: a component pushes at most its adjacency entries plus its root
    if (tid == 0) sh_tot = 0;
    __syncthreads();
    for (int base = 0; base < K; base += nt) {
        const int k = base + tid;
        const int v = k < K ? deg[uf_root(par, list[k])] + 1 : 0;
        int tot;
        const int pos = block_excl(v, ws, &tot);
        const int c0 = sh_tot;
        if (k < K) stk_off[k] = c0 + pos;
        __syncthreads();
        if (tid == 0) sh_tot = c0 + tot;
        __syncthreads();
    }
    int* stack_base = d.stack + 2 * (x.e0 + (x.joints ? d.je.world_start[x.w] : 0)) + x.s;
    // count
    for (int k = tid; k < K; k += nt) {
        int r, b, sy;
        bool ready, joint;
        const int cap = deg[uf_root(par, list[k])] + 1;
        island_search<true>(d, x, list[k], stack_base + stk_off[k], cap, 0, 0, 0, false, x.s + k, &r, &b, &sy, &ready, &joint);
        const bool sleeps = x.may_sleep && ready;
        kind[k] = sleeps ? 2 : (r > 0 ? 1 : 0);
        n_rows[k] = kind[k] == 1 ? r : 0;
        n_bod[k] = kind[k] == 1 ? b : 0;
        n_sys[k] = kind[k] == 1 ? sy : 0;
        o_sys[k] = joint ? 1 : 0;   // island flags until the prefix below
    }
    __syncthreads();
    // prefixes in component order: rows, bodies, systems, island index
    __shared__ int c_rows, c_bod, c_sys, c_isl;
    if (tid == 0) { c_rows = row0; c_bod = x.s; c_sys = sys0; c_isl = 0; }
    __syncthreads();
    for (int base = 0; base < K; base += nt) {
        const int k = base + tid;
        const bool in = k < K;
        int t1, t2, t3, t4;
        const int pr = block_excl(in ? n_rows[k] : 0, ws, &t1);
        const int pb = block_excl(in ? n_bod[k] : 0, ws, &t2);
        const int psy = block_excl(in ? n_sys[k] : 0, ws, &t3);
        const int pi = block_excl(in && kind[k] == 1 ? 1 : 0, ws, &t4);
        if (in) {
            const int flag = o_sys[k];
            o_rows[k] = c_rows + pr;
            o_bod[k] = c_bod + pb;
            o_sys[k] = c_sys + psy;
            if (kind[k] == 1) {
                const int ii = x.s + c_isl + pi;
                d.isl_row_start[ii] = c_rows + pr;
                d.isl_row_count[ii] = n_rows[k];
                d.isl_body_start[ii] = c_bod + pb;
                d.isl_body_count[ii] = n_bod[k];
                d.isl_world[ii] = x.w;
                if (x.joints) {
                    d.isl_flags[ii] = flag;
                    d.isl_sys_start[ii] = c_sys + psy;
                    d.isl_sys_count[ii] = n_sys[k];
                }
            }
        }
        __syncthreads();
        if (tid == 0) { c_rows += t1; c_bod += t2; c_sys += t3; c_isl += t4; }
        __syncthreads();
    }
    // write (the count marked the searched bodies -2, which the write pass
    // treats as not visited)
    for (int k = tid; k < K; k += nt) {
        if (kind[k] == 0) continue;
        const int cap = deg[uf_root(par, list[k])] + 1;
        island_search<false>(d, x, list[k], stack_base + stk_off[k], cap, o_rows[k], o_bod[k], o_sys[k], kind[k] == 2, 0,
                             nullptr, nullptr, nullptr, nullptr, nullptr);
    }
    __syncthreads();
    if (tid == 0) {
        d.isl_count_w[x.w] = c_isl;
        *sh_rows_end = c_rows;
    }
}

__global__ void __launch_bounds__(256) k_islands(Dev d, int smem_bytes) {
    extern __shared__ int sm_isl[];
    __shared__ int sh_carry, sh_rows_end;
    __shared__ int warp_sums[8];
    const int w = blockIdx.x;
    const int s = d.world_start[w], e = d.world_start[w + 1];
    const int ne = *d.n_edges_new, ncon = *d.n_contacts_new;
    const int e0 = lower_bound_u64(d.e_new.key, ne, (uint64_t)s << 32);
    const int e1 = lower_bound_u64(d.e_new.key, ne, (uint64_t)e << 32);
    const int c0 = (e0 < ne) ? d.e_new.cstart[e0] : ncon;
    const int c1 = (e1 < ne) ? d.e_new.cstart[e1] : ncon;
    // joint edges and joints of this world (row slots of the world start after
    // the joints of the worlds before it)
    const bool joints = d.n_joint_edges > 0;
    const int je0 = joints ? d.je.world_start[w] : 0, je1 = joints ? d.je.world_start[w + 1] : 0;
    const int jj0 = joints ? d.je.world_jstart[w] : 0;
    const int sys0 = joints ? d.hs_world_start[w] : 0;
    const int nb = e - s, ne_w = e1 - e0, nj = je1 - je0, E = ne_w + nj;
    const int stack_cap = 2 * E + nb;
    const bool fast = islands_need(nb, ne_w, nj) <= smem_bytes;
    int *vis, *a_ofs, *a_cur, *adj, *live, *stk, *order = nullptr;
    const uint8_t* mov;
    uint8_t* mov_s = nullptr;
    if (fast) {
        vis = sm_isl; a_ofs = vis + nb; a_cur = a_ofs + nb; adj = a_cur + nb;
        live = adj + 4 * E; stk = live + ne_w; order = stk + stack_cap;
        mov_s = reinterpret_cast<uint8_t*>(order + nb);
        mov = mov_s;
    } else {
        vis = d.visited + s; a_ofs = d.adj_ofs + s; a_cur = d.adj_cursor + s;
        adj = d.adj_list + 4 * (size_t)(e0 + je0);   // entries from 2 (e0 + je0), two ints each
        live = d.edge_live + e0;
        stk = d.stack + 2 * (e0 + je0) + s;
        mov = d.movement + s;
    }
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < nb; i += nt) {
        a_cur[i] = 0;
        vis[i] = -1;
        if (fast) { mov_s[i] = d.movement[s + i]; order[i] = d.map_order[s + i] - s; }
    }
    for (int c = c0 + tid; c < c1; c += nt) d.row_of_contact[c] = -1;
    // live contacts per edge, so that the serial DFS below advances its row
    // cursor by one load per edge instead of one per contact
    for (int k = tid; k < ne_w; k += nt) {
        const int cs = d.e_new.cstart[e0 + k], cn = d.e_new.ccount[e0 + k];
        int l = 0;
        for (int c = cs; c < cs + cn; c++) l += cs_live(d.c_new.state[c]);
        live[k] = l;
        d.edge_row[e0 + k] = -1;
    }
    __syncthreads();
    for (int k = tid; k < ne_w; k += nt) {
        const uint64_t key = d.e_new.key[e0 + k];
        const int a = (int)(key >> 32) - s, b = (int)(key & 0xffffffffu) - s;
        if (mov[a] == 0) atomicAdd(&a_cur[a], 1);
        if (mov[b] == 0) atomicAdd(&a_cur[b], 1);
    }
    for (int k = tid; k < nj; k += nt) {
        const uint64_t key = d.je.key[je0 + k];
        const int a = (int)(key >> 32) - s, b = (int)(key & 0xffffffffu) - s;
        if (mov[a] == 0) atomicAdd(&a_cur[a], 1);
        if (mov[b] == 0) atomicAdd(&a_cur[b], 1);
    }
    __syncthreads();
    // exclusive scan of the degrees into adjacency offsets
    if (tid == 0) sh_carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += nt) {
        const int i = base + tid;
        const int v = (i < nb) ? a_cur[i] : 0;
        int x = v;
        const int lane = tid & 31, wid = tid >> 5;
        for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += t; }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int y = (lane < (nt >> 5)) ? warp_sums[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, y, o); if (lane >= o) y += t; }
            if (lane < 8) warp_sums[lane] = y;
        }
        __syncthreads();
        const int incl = x + (wid > 0 ? warp_sums[wid - 1] : 0);
        const int carry = sh_carry;
        if (i < nb) { a_ofs[i] = carry + incl - v; a_cur[i] = carry + incl - v; }
        __syncthreads();
        if (tid == nt - 1) sh_carry = carry + incl;
        __syncthreads();
    }
    for (int k = tid; k < ne_w; k += nt) {
        const uint64_t key = d.e_new.key[e0 + k];
        const int a = (int)(key >> 32) - s, b = (int)(key & 0xffffffffu) - s;
        if (mov[a] == 0) { int slot = atomicAdd(&a_cur[a], 1); adj[2 * slot] = b; adj[2 * slot + 1] = k; }
        if (mov[b] == 0) { int slot = atomicAdd(&a_cur[b], 1); adj[2 * slot] = a; adj[2 * slot + 1] = k; }
    }
    __syncthreads();
    // joint edges after the contact edges, marked -(index + 1); the sort below
    // is stable, so a pair holding both kinds lists its contacts first
    for (int k = tid; k < nj; k += nt) {
        const uint64_t key = d.je.key[je0 + k];
        const int a = (int)(key >> 32) - s, b = (int)(key & 0xffffffffu) - s;
        if (mov[a] == 0) { int slot = atomicAdd(&a_cur[a], 1); adj[2 * slot] = b; adj[2 * slot + 1] = -(je0 + k + 1); }
        if (mov[b] == 0) { int slot = atomicAdd(&a_cur[b], 1); adj[2 * slot] = a; adj[2 * slot + 1] = -(je0 + k + 1); }
    }
    __syncthreads();
    // each dynamic node's edges sorted by the other body's id (insertion sort)
    for (int i = tid; i < nb; i += nt) {
        if (mov[i] != 0) continue;
        const int lo = a_ofs[i], hi = a_cur[i];
        for (int x = lo + 1; x < hi; x++) {
            const int ko = adj[2 * x], kk = adj[2 * x + 1];
            int y = x - 1;
            while (y >= lo && adj[2 * y] > ko) { adj[2 * (y + 1)] = adj[2 * y]; adj[2 * (y + 1) + 1] = adj[2 * y + 1]; y--; }
            adj[2 * (y + 1)] = ko;
            adj[2 * (y + 1) + 1] = kk;
        }
    }
    __syncthreads();
    if (d.comp != nullptr && nb > kTileWorld) {
        IslandCtx x;
        x.w = w; x.s = s; x.e0 = e0; x.ready_steps = d.wparams[w].ready_steps;
        x.sleep_on = d.has_sleep != 0;
        x.may_sleep = x.sleep_on && d.wparams[w].sleeping;
        x.joints = joints;
        x.a_ofs = a_ofs; x.a_cur = a_cur; x.adj = adj; x.live = live; x.mov = mov; x.vis = vis;
        islands_big(d, x, nb, c0 + jj0, sys0, warp_sums, &sh_rows_end);
    } else if (tid == 0) {
        // sleeping (sleepOrSolveIslands, PhysicsEngine.cpp:1536-1613): a
        // sleeping body's edges to sleeping or fixed bodies carry no rows, and
        // an island whose bodies are all ready to sleep (and touch no
        // kinematic body) falls asleep instead of being solved
        const bool sleep_on = d.has_sleep != 0;                 // sleeping bodies may exist
        const bool may_sleep = sleep_on && d.wparams[w].sleeping;   // islands may fall asleep
        const int ready_steps = d.wparams[w].ready_steps;
        int rc = c0 + jj0, bc = s, ni = 0, sc = sys0;
        for (int t = s; t < e; t++) {
            const int node = fast ? order[t - s] : d.map_order[t] - s;
            if (mov[node] != 0 || vis[node] >= 0) continue;
            const int rs = rc, bs = bc, ss = sc;
            int sp = 0;
            bool has_joint = false, all_ready = true;
            stk[sp++] = node;
            while (sp > 0) {
                const int cur = stk[--sp];
                if (vis[cur] >= 0) continue;
                vis[cur] = bc - bs;
                d.isl_bodies[bc++] = cur + s;
                const int lo = a_ofs[cur], hi = a_cur[cur];
                const bool cur_asleep = sleep_on && d.asleep[cur + s];
                bool kinematic_contact = false;
                // each edge to a not-yet-visited neighbour emits its rows, then
                // the neighbour (if dynamic) is pushed; visits happen only at
                // pops, so one pass over the edges gives the rows in edge order
                // and the pushes in edge order
                for (int j = lo; j < hi; j++) {
                    const int o = adj[2 * j], k = adj[2 * j + 1];
                    if (mov[o] == 2) kinematic_contact = true;
                    if (vis[o] >= 0) continue;
                    if (cur_asleep && (mov[o] == 1 || d.asleep[o + s])) {
                        // no rows; the neighbour still joins the island
                    } else if (k < 0) {
                        // joint edge: its holonomic system joins the island's
                        // list at first sight, then its joints' rows
                        const int je = -k - 1, sy = d.je.sys[je];
                        if (sy >= 0) {
                            bool seen = false;
                            for (int q = ss; q < sc; q++) seen |= d.isl_sys[q] == sy;
                            if (!seen) d.isl_sys[sc++] = sy;
                        }
                        // the edge's joints in creation order; a cone or
                        // twist limit only while its last rebuild found the
                        // limit reached (ConeRotationLimit::addSolverConstraints,
                        // PersistentConstraint.h:165, 205); a spring-only
                        // edge emits no rows
                        for (int q = d.je.jstart[je]; q < d.je.jstart[je] + d.je.jcount[je]; q++) {
                            const int jj = d.je.jlist[q];
                            if (jk_conditional(d.jt.kind[jj]) && !d.jt.active[jj]) continue;
                            d.row_contact[rc++] = -(jj + 1);
                            has_joint = true;
                        }
                    } else {
                        // the edge's live contacts take the next rows (written below)
                        const int nl = live[k];
                        if (nl > 0) { d.edge_row[e0 + k] = rc; rc += nl; }
                    }
                    if (mov[o] == 0) {
                        if (sp < stack_cap) stk[sp++] = o;
                        else atomicOr(d.status, ST_STACK_OVERFLOW);
                    }
                }
                if (may_sleep && (kinematic_contact || d.ready_cnt[cur + s] < ready_steps)) all_ready = false;
            }
            if (may_sleep && all_ready) {
                // the island falls asleep (RigidBody::sleep): zero velocities,
                // its rows and systems are dropped, its edges' row slots freed
                for (int q = bs; q < bc; q++) {
                    const int g = d.isl_bodies[q];
                    d.asleep[g] = 1;
                    d.vel[g] = make_float4(0.f, 0.f, 0.f, 0.f);
                    d.angv[g] = make_float4(0.f, 0.f, 0.f, 0.f);
                    const int lb = g - s;
                    for (int j = a_ofs[lb]; j < a_cur[lb]; j++) {
                        const int k = adj[2 * j + 1];
                        if (k >= 0 && d.edge_row[e0 + k] >= rs) d.edge_row[e0 + k] = -1;
                    }
                }
                rc = rs;
                bc = bs;
                sc = ss;
                continue;
            }
            if (rc > rs) {
                d.isl_row_start[s + ni] = rs;
                d.isl_row_count[s + ni] = rc - rs;
                d.isl_body_start[s + ni] = bs;
                d.isl_body_count[s + ni] = bc - bs;
                d.isl_world[s + ni] = w;
                if (joints) {
                    d.isl_flags[s + ni] = has_joint ? 1 : 0;
                    d.isl_sys_start[s + ni] = ss;
                    d.isl_sys_count[s + ni] = sc - ss;
                }
                ni++;
            } else {
                bc = bs;
                sc = ss;
            }
        }
        d.isl_count_w[w] = ni;
        sh_rows_end = rc;
    }
    __syncthreads();
    if (fast)
        for (int i = tid; i < nb; i += nt) d.visited[s + i] = vis[i];
    // each emitted edge's live contacts into its rows, in contact order
    for (int k = e0 + tid; k < e1; k += nt) {
        int r = d.edge_row[k];
        if (r < 0) continue;
        const int cs = d.e_new.cstart[k], cn = d.e_new.ccount[k];
        for (int c = cs; c < cs + cn; c++)
            if (cs_live(d.c_new.state[c])) d.row_contact[r++] = c;
    }
    __syncthreads();
    const int rows_end = sh_rows_end;
    for (int r = c0 + jj0 + tid; r < rows_end; r += nt) {
        int c = d.row_contact[r];
        if (c < 0) {
            const int j = -c - 1, a = d.jt.b1[j], b = d.jt.b2[j];
            d.jt.rows[j].sa = (d.movement[a] == 0) ? d.visited[a] : -1;
            d.jt.rows[j].sb = (d.movement[b] == 0) ? d.visited[b] : -1;
            d.rows[r].contact = c;
            continue;
        }
        d.row_of_contact[c] = r;
        uint64_t key = d.e_new.key[d.c_new.edge[c]];
        int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
        d.rows[r].sa = (d.movement[a] == 0) ? d.visited[a] : -1;
        d.rows[r].sb = (d.movement[b] == 0) ? d.visited[b] : -1;
        d.rows[r].contact = c;
    }
}

__global__ void k_island_copy(Dev d) {
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < d.n_worlds; w += gridDim.x * blockDim.x) {
        int s = d.world_start[w], n = d.isl_count_w[w], o = d.isl_scan[w];
        for (int k = 0; k < n; k++) {
            d.g_isl_row_start[o + k] = d.isl_row_start[s + k];
            d.g_isl_row_count[o + k] = d.isl_row_count[s + k];
            d.g_isl_body_start[o + k] = d.isl_body_start[s + k];
            d.g_isl_body_count[o + k] = d.isl_body_count[s + k];
            d.g_isl_world[o + k] = d.isl_world[s + k];
            if (d.n_joint_edges > 0) {
                d.g_isl_flags[o + k] = d.isl_flags[s + k];
                d.g_isl_sys_start[o + k] = d.isl_sys_start[s + k];
                d.g_isl_sys_count[o + k] = d.isl_sys_count[s + k];
            }
        }
    }
}

int grid_for(int n, int per_block, int n_sms) {
    int g = (n + per_block - 1) / per_block;
    int cap = n_sms * 8;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

}  // namespace

void launch_merge(const Dev& d, const Launch& L) {
    const int gb = L.n_sms * 4, bs = 256;
    int* cnt = d.cnt;
    k_surv<<<gb, bs, 0, L.st>>>(d);
    scan_exclusive(d.surv, d.surv_scan, d.n_edges_old, 0, d.cap_edges, cnt + 0, d.scan_tmp, L);
    k_pair_match<<<gb, bs, 0, L.st>>>(d);
    scan_exclusive(d.unm, d.unm_scan, d.n_pairs, 0, d.cap_pairs, cnt + 1, d.scan_tmp, L);
    k_place<<<gb, bs, 0, L.st>>>(d, cnt);
    k_edge_total<<<1, 1, 0, L.st>>>(d, cnt);
    k_contacts<<<gb, 128, 0, L.st>>>(d, 0);
    scan_exclusive(d.edge_cnt, d.e_new.cstart, d.n_edges_new, 0, d.cap_edges, d.n_contacts_new, d.scan_tmp, L);
    k_contact_total<<<1, 1, 0, L.st>>>(d);
    k_contacts<<<gb, 128, 0, L.st>>>(d, 1);
}

// Edge and contact index ranges of the given worlds in the current contact
// graph (edges sorted by key, contacts stored in edge order): out[4 w] =
// (first edge, end edge, first contact, end contact).
__global__ void k_world_ranges(const uint64_t* keys, const int* cstart, const int* n_edges, const int* n_contacts,
                               const int* world_start, const int* worlds, int n, int* out) {
    const int ne = *n_edges, nc = *n_contacts;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int w = worlds[i];
        const int e0 = lower_bound_u64(keys, ne, (uint64_t)world_start[w] << 32);
        const int e1 = lower_bound_u64(keys, ne, (uint64_t)world_start[w + 1] << 32);
        out[4 * i] = e0;
        out[4 * i + 1] = e1;
        out[4 * i + 2] = e0 < ne ? cstart[e0] : nc;
        out[4 * i + 3] = e1 < ne ? cstart[e1] : nc;
    }
}

void launch_world_ranges(const Dev& d, const int* worlds, int n, int* out, cudaStream_t st) {
    k_world_ranges<<<(n + 127) / 128, 128, 0, st>>>(d.e_old.key, d.e_old.cstart, d.n_edges_old, d.n_contacts_old, d.world_start,
                                                      worlds, n, out);
}

int islands_smem_bytes(int max_bodies) {
    // about four constraint edges per body, at most kIslandsSmemMax; the
    // kernel's limit (shared by every batch of the process) is that maximum
    const long long want = 4LL * (6LL * max_bodies + 7LL * 4 * max_bodies) + max_bodies + 64;
    cudaFuncSetAttribute(k_islands, cudaFuncAttributeMaxDynamicSharedMemorySize, kIslandsSmemMax);
    return (int)std::min<long long>(want, kIslandsSmemMax);
}

void launch_islands(const Dev& d, int smem_bytes, const Launch& L) {
    k_islands<<<d.n_worlds, 256, smem_bytes, L.st>>>(d, smem_bytes);
    scan_exclusive(d.isl_count_w, d.isl_scan, nullptr, d.n_worlds, d.n_worlds, d.n_islands, d.scan_tmp, L);
    k_island_copy<<<grid_for(d.n_worlds, 128, L.n_sms), 128, 0, L.st>>>(d);
}

}  // namespace cpgpu
