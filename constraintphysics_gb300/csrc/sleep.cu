// sleep.cu — the start of a step when sleeping is enabled: waking actions,
// the sleep bookkeeping and gravity (PhysicsEngine.cpp:65-87;
// RigidBody::recordMovementState, RigidBody.cpp:347-352; bodySleepy,
// PhysicsEngine.cpp:1221-1254).
//
// Per body, in creation order: a body that received a waking action (an API
// setter or a spring impulse since the last step) wakes its island -- every
// sleeping dynamic body connected to it through dynamic bodies by an edge of
// the constraint graph (wakeupIsland, PhysicsEngine.cpp:1263-1283); then an
// awake dynamic body records its velocities (the last sleep_delay / dt steps),
// counts the step as sleepy or not, and takes gravity.  Wakes can reset the
// records of bodies already handled this step, so a world with any waking
// body is handled by one thread in body order (its graph's components from a
// union-find over the edges between dynamic bodies); the other worlds' bodies
// are independent and run in parallel.
#include "kernels.cuh"
#include "devmath.cuh"

namespace cpgpu {

namespace {

__device__ __forceinline__ int lower_bound_key(const uint64_t* keys, int n, uint64_t k) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (keys[m] < k) lo = m + 1; else hi = m;
    }
    return lo;
}

// union-find over the world's bodies (world-local indices) in `par`
__device__ int uf_find(int* par, int x) {
    while (par[x] != x) {
        par[x] = par[par[x]];
        x = par[x];
    }
    return x;
}
__device__ void uf_union(int* par, int a, int b) {
    a = uf_find(par, a);
    b = uf_find(par, b);
    if (a != b) par[a < b ? b : a] = a < b ? a : b;
}

// RigidBody::recordMovementState and the sleepy count of one awake dynamic
// body, then gravity
__device__ void record_body(const Dev& d, const WorldParams& P, int i) {
    float4 v = d.vel[i];
    const float4 w = d.angv[i];
    const int len = P.hist_len > 0 ? P.hist_len : 1;
    float* h = d.hist + (size_t)d.hist_cap * 6 * i;
    int n = d.hist_n[i], head = d.hist_head[i];
    int slot;
    if (n < len) { slot = (head + n) % len; n++; }
    else { slot = head; head = (head + 1) % len; }
    h[6 * slot + 0] = v.x; h[6 * slot + 1] = v.y; h[6 * slot + 2] = v.z;
    h[6 * slot + 3] = w.x; h[6 * slot + 4] = w.y; h[6 * slot + 5] = w.z;
    d.hist_n[i] = n;
    d.hist_head[i] = head;
    bool sleepy = false;
    if (n >= P.hist_min && n >= 2) {
        f3 av = mk(0.f, 0.f, 0.f), aw = mk(0.f, 0.f, 0.f);
        for (int k = 0; k < n; k++) {
            const float* e = h + 6 * ((head + k) % len);
            av = av + mk(e[0], e[1], e[2]);
            aw = aw + mk(e[3], e[4], e[5]);
        }
        av = av * (1.0f / (float)n);
        aw = aw * (1.0f / (float)n);
        const float* first = h + 6 * head;
        const float* last = h + 6 * ((head + n - 1) % len);
        const float span = P.dt * (float)(n - 1);
        const f3 acc = (mk(last[0], last[1], last[2]) - mk(first[0], first[1], first[2])) * (1.0f / span);
        const f3 aacc = (mk(last[3], last[4], last[5]) - mk(first[3], first[4], first[5])) * (1.0f / span);
        sleepy = mag(av) <= P.vel_eps && mag(aw) <= P.ang_vel_eps && mag(acc) <= P.accel_eps && mag(aacc) <= P.ang_accel_eps;
    }
    if (sleepy) {
        if (d.ready_cnt[i] < (1 << 30)) d.ready_cnt[i] += 1;
    } else {
        const int ns = d.non_sleepy[i] + 1;
        if (ns >= P.non_sleepy_threshold) { d.ready_cnt[i] = 0; d.non_sleepy[i] = 0; }
        else d.non_sleepy[i] = ns;
    }
    v.x += P.gx * P.dt; v.y += P.gy * P.dt; v.z += P.gz * P.dt;
    d.vel[i] = v;
}

// RigidBody::wake for every sleeping dynamic body of component `c`
__device__ void wake_component(const Dev& d, int* par, int s, int e, int c) {
    for (int j = s; j < e; j++) {
        if (d.movement[j] != 0 || !d.asleep[j] || uf_find(par, j - s) != c) continue;
        d.asleep[j] = 0;
        d.ready_cnt[j] = 0;
        d.non_sleepy[j] = 0;
        d.hist_n[j] = 0;
        d.hist_head[j] = 0;
    }
}

__global__ void __launch_bounds__(128) k_sleep_begin(Dev d) {
    for (int w = blockIdx.x; w < d.n_worlds; w += gridDim.x) {
        const WorldParams& P = d.wparams[w];
        const int s = d.world_start[w], e = d.world_start[w + 1];
        int any = 0;
        for (int i = s + threadIdx.x; i < e; i += blockDim.x) any |= d.waking[i];
        any = __syncthreads_or(any);
        if (!any) {
            for (int i = s + threadIdx.x; i < e; i += blockDim.x)
                if (d.movement[i] == 0 && !d.asleep[i]) record_body(d, P, i);
        } else if (threadIdx.x == 0) {
            // components of the graph at the start of the step: contact edges
            // with a contact that has not expired, and joint / spring edges
            int* par = d.visited + s;
            for (int i = 0; i < e - s; i++) par[i] = i;
            const int ne = *d.n_edges_old;
            const int e0 = lower_bound_key(d.e_old.key, ne, (uint64_t)s << 32);
            const int e1 = lower_bound_key(d.e_old.key, ne, (uint64_t)e << 32);
            auto edge_alive = [&](int k) {
                for (int c = d.e_old.cstart[k]; c < d.e_old.cstart[k] + d.e_old.ccount[k]; c++)
                    if (!cs_dead(d.c_old.state[c])) return true;
                return false;
            };
            for (int k = e0; k < e1; k++) {
                const uint64_t key = d.e_old.key[k];
                const int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
                if (d.movement[a] == 0 && d.movement[b] == 0 && edge_alive(k)) uf_union(par, a - s, b - s);
            }
            const int je0 = d.n_joint_edges > 0 ? d.je.world_start[w] : 0, je1 = d.n_joint_edges > 0 ? d.je.world_start[w + 1] : 0;
            for (int k = je0; k < je1; k++) {
                const uint64_t key = d.je.key[k];
                const int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
                if (d.movement[a] == 0 && d.movement[b] == 0) uf_union(par, a - s, b - s);
            }
            for (int i = s; i < e; i++) {
                if (d.waking[i]) {
                    d.waking[i] = 0;
                    if (d.movement[i] == 0) {
                        wake_component(d, par, s, e, uf_find(par, i - s));
                    } else {
                        // a fixed or kinematic body wakes the islands of its
                        // dynamic neighbours
                        for (int k = e0; k < e1; k++) {
                            const uint64_t key = d.e_old.key[k];
                            const int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
                            const int o = a == i ? b : (b == i ? a : -1);
                            if (o >= 0 && d.movement[o] == 0 && edge_alive(k)) wake_component(d, par, s, e, uf_find(par, o - s));
                        }
                        for (int k = je0; k < je1; k++) {
                            const uint64_t key = d.je.key[k];
                            const int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
                            const int o = a == i ? b : (b == i ? a : -1);
                            if (o >= 0 && d.movement[o] == 0) wake_component(d, par, s, e, uf_find(par, o - s));
                        }
                    }
                }
                if (d.movement[i] == 0 && !d.asleep[i]) record_body(d, P, i);
            }
        }
        __syncthreads();
    }
}

}  // namespace

void launch_step_begin(const Dev& d, const Launch& L) {
    if (!d.has_sleep) { launch_gravity(d, L); return; }
    int g = d.n_worlds < L.n_sms * 16 ? d.n_worlds : L.n_sms * 16;
    k_sleep_begin<<<g < 1 ? 1 : g, 128, 0, L.st>>>(d);
}

}  // namespace cpgpu
