// cluster.cu - pose clustering of matchScene (ppf.cpp:414-418): sortPoses, clusterPose,
// avgClusters, sortPoses, clusterPose2 (util.cpp:486-601).
//
// One CTA. The sorts are stable rank-by-counting sorts on (votes desc, list position).
// The two greedy first-fit clusterings are sequential by definition (a pose joins the
// first earlier cluster head it is compatible with); warp 0 walks the poses in order and
// tests the current heads 32 at a time with a ballot. Sums run in member order, so the
// result is identical to the oracle's sequential restatement.
#include "sm_icp.h"
#include "sm_stages.h"

namespace sm {

namespace {

constexpr int kClBs = 1024;
constexpr int PF    = smi::kPoseFloats;

__device__ __forceinline__ float norm3(float x, float y, float z) {
    return smm::fsqrt(x * x + (y * y + z * z));
}

// out[rank(i)] = in[i] for the stable sort by votes (float 17) descending.
__device__ void stable_sort_votes(const float *in, int n, float *out) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float v    = in[(size_t)i * PF + 17];
        int         rank = 0;
        for (int j = 0; j < n; j++) {
            const float u = in[(size_t)j * PF + 17];
            rank += (u > v || (u == v && j < i)) ? 1 : 0;
        }
        for (int e = 0; e < PF; e++)
            out[(size_t)rank * PF + e] = in[(size_t)i * PF + e];
    }
}

struct ClArgs {
    const float *poses;
    int          np;
    float        distThr, angThr, cx, cy, cz, thr2;
    float       *sorted;  // np x PF
    int         *clu, *next, *tail, *heads; // np each
    float       *avg;     // np x PF (cluster creation order)
    float       *avgSorted;
    float4      *tr;      // np
    int         *lead2;   // np
    float       *out;     // np x PF
    int         *outCount;
};

__global__ void __launch_bounds__(kClBs) k_cluster(ClArgs a) {
    __shared__ int sNh, sNout;
    const int      tid = threadIdx.x, lane = tid & 31;
    const int      np  = a.np;
    stable_sort_votes(a.poses, np, a.sorted);
    __syncthreads();
    // clusterPose: warp 0 walks the poses in sorted order
    if (tid < 32) {
        int nh = 0;
        for (int i = 0; i < np; i++) {
            const float *P     = a.sorted + (size_t)i * PF;
            const float  tx = P[3], ty = P[7], tz = P[11], an = P[16];
            int          found = -1;
            for (int h0 = 0; h0 < nh && found < 0; h0 += 32) {
                const int h  = h0 + lane;
                bool      ok = false;
                if (h < nh) {
                    const float *H = a.sorted + (size_t)a.heads[h] * PF;
                    const float  d = norm3(tx - H[3], ty - H[7], tz - H[11]);
                    ok             = d < a.distThr && smm::fabs_(an - H[16]) < a.angThr;
                }
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (m)
                    found = h0 + __ffs(m) - 1;
            }
            if (lane == 0) {
                a.next[i] = -1;
                if (found < 0) {
                    a.heads[nh] = i;
                    a.clu[i]    = nh;
                    a.tail[nh]  = i;
                } else {
                    a.clu[i]              = found;
                    a.next[a.tail[found]] = i;
                    a.tail[found]         = i;
                }
            }
            if (found < 0)
                nh++;
            __syncwarp();
        }
        if (lane == 0)
            sNh = nh;
    }
    __syncthreads();
    const int nh = sNh;
    // avgClusters: mean translation, summed votes, Markley quaternion average
    for (int h = tid; h < nh; h += kClBs) {
        float  px = 0.f, py = 0.f, pz = 0.f, votes = 0.f;
        double S[10];
        for (int e = 0; e < 10; e++)
            S[e] = 0.0;
        int cnt = 0;
        for (int i = a.heads[h]; i >= 0; i = a.next[i]) {
            const float *P = a.sorted + (size_t)i * PF;
            px             = px + P[3];
            py             = py + P[7];
            pz             = pz + P[11];
            votes          = votes + P[17];
            const double v[4] = {P[12], P[13], P[14], P[15]};
            int          k    = 0;
            for (int r = 0; r < 4; r++)
                for (int s = r; s < 4; s++)
                    S[k++] += v[r] * v[s];
            cnt++;
        }
        double q[4], R[9];
        sml::quat_average_from_sum(S, cnt, q);
        sml::quat_to_mat(q, R);
        float *O = a.avg + (size_t)h * PF;
        for (int r = 0; r < 3; r++)
            for (int s = 0; s < 3; s++)
                O[r * 4 + s] = (float)R[r * 3 + s];
        const float fc = (float)cnt;
        O[3]           = smm::fdiv(px, fc);
        O[7]           = smm::fdiv(py, fc);
        O[11]          = smm::fdiv(pz, fc);
        for (int r = 0; r < 4; r++)
            O[12 + r] = (float)q[r];
        O[16] = sml::quat_angle(q);
        O[17] = votes;
    }
    __syncthreads();
    stable_sort_votes(a.avg, nh, a.avgSorted);
    __syncthreads();
    // clusterPose2: overlap of the transformed model-box centres
    for (int h = tid; h < nh; h += kClBs) {
        smi::Pose34 T;
        for (int e = 0; e < 12; e++)
            T.m[e] = a.avgSorted[(size_t)h * PF + e];
        float x, y, z;
        smi::pose_apply(T, a.cx, a.cy, a.cz, x, y, z);
        a.tr[h] = make_float4(x, y, z, 0.f);
    }
    __syncthreads();
    if (tid < 32) {
        int nl = 0;
        for (int i = 0; i < nh; i++) {
            const float4 ti    = a.tr[i];
            int          found = -1;
            for (int h0 = 0; h0 < nl && found < 0; h0 += 32) {
                const int h  = h0 + lane;
                bool      ok = false;
                if (h < nl) {
                    const float4 th = a.tr[a.heads[h]];
                    const float  dx = th.x - ti.x, dy = th.y - ti.y, dz = th.z - ti.z;
                    ok              = dx * dx + (dy * dy + dz * dz) < a.thr2;
                }
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (m)
                    found = h0 + __ffs(m) - 1;
            }
            if (lane == 0) {
                if (found < 0) {
                    a.heads[nl] = i; // heads[] reused: leaders of clusterPose2
                    float *O    = a.out + (size_t)nl * PF;
                    for (int e = 0; e < PF; e++)
                        O[e] = a.avgSorted[(size_t)i * PF + e];
                } else {
                    float *O = a.out + (size_t)found * PF;
                    O[17]    = O[17] + a.avgSorted[(size_t)i * PF + 17];
                }
            }
            if (found < 0)
                nl++;
            __syncwarp();
        }
        if (lane == 0)
            sNout = nl;
    }
    __syncthreads();
    if (tid == 0)
        *a.outCount = sNout;
}

} // namespace

int cluster(Ctx &c, const float *poses, int np, float distThr, float angThr, const float center[3],
            float maxOverlap, float *outCands, const std::string &tag) {
    if (np <= 0)
        return 0;
    ClArgs a;
    a.poses     = poses;
    a.np        = np;
    a.distThr   = distThr;
    a.angThr    = angThr;
    a.cx        = center[0];
    a.cy        = center[1];
    a.cz        = center[2];
    a.thr2      = maxOverlap * maxOverlap;
    a.sorted    = c.arena.get<float>(tag + ".sorted", (size_t)np * PF);
    int *ib     = c.arena.get<int>(tag + ".ints", (size_t)np * 5 + 1);
    a.clu       = ib;
    a.next      = ib + np;
    a.tail      = ib + 2 * np;
    a.heads     = ib + 3 * np;
    a.lead2     = ib + 4 * np;
    a.outCount  = ib + 5 * np;
    a.avg       = c.arena.get<float>(tag + ".avg", (size_t)np * PF);
    a.avgSorted = c.arena.get<float>(tag + ".avgs", (size_t)np * PF);
    a.tr        = c.arena.get<float4>(tag + ".tr", np);
    a.out       = outCands;
    k_cluster<<<1, kClBs, 0, c.stream>>>(a);
    SM_LAUNCH_CHECK();
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, a.outCount, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    return c.hostCounts[0];
}

} // namespace sm
