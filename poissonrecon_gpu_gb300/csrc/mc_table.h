// Marching-cubes case tables, generated at start-up from first principles.
//
// Conventions follow the reference pipeline (MarchingCubes.cuh:693-744 and the
// VertexIndex/edgeVertex usage in main.cu:2444-2582):
//   * cube vertex v in 0..7 sits at (x,y,z) = (0,0,0),(1,0,0),(1,1,0),(0,1,0),
//     (0,0,1),(1,0,1),(1,1,1),(0,1,1);
//   * edge e in 0..11 has orientation e>>2 (0=x,1=y,2=z); bits e&1 and (e>>1)&1
//     give the offsets along the two remaining axes in increasing axis order;
//   * the case index sets bit v when the value at vertex v is negative.
// Polygons are traced across the six faces.  On a face whose four corners
// alternate in sign the negative corners are kept apart, which is the rule
// that reproduces the reference table's triangle count and edge set for all
// 256 cases.  Each polygon is oriented so that its normal points from the
// negative side to the positive side and is triangulated as a fan.
#pragma once
#include <cstring>

namespace prgpu_mc {

struct Tables {
    int tri_count[256];      // triangles per case
    int tri_edges[256][16];  // 3*tri_count edge ids, -1 padded
    int edge_v[12][2];       // endpoint vertices of each edge (interpolation order)
};

inline void vertex_xyz(int v, int p[3]) {
    static const int X[8] = {0, 1, 1, 0, 0, 1, 1, 0};
    static const int Y[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    static const int Z[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    p[0] = X[v]; p[1] = Y[v]; p[2] = Z[v];
}

inline int vertex_id(int x, int y, int z) {
    int r = x | (z << 2);
    if (y) r += (r & 1) ? 1 : 3;
    return r;
}

// Endpoints of edge e: the end with the smaller coordinate along the edge
// first, except x-edges on the y=1 side, which the reference lists from the
// x=1 end (edgeVertex rows 1 and 3).
inline void edge_endpoints(int e, int out[2]) {
    int o = e >> 2;
    int a0 = (o == 0) ? 1 : 0, a1 = (o == 2) ? 1 : 2;
    int p[3] = {0, 0, 0};
    p[a0] = e & 1;
    p[a1] = (e >> 1) & 1;
    int q[3] = {p[0], p[1], p[2]};
    q[o] = 1;
    int v0 = vertex_id(p[0], p[1], p[2]), v1 = vertex_id(q[0], q[1], q[2]);
    if (o == 0 && p[1] == 1) { int t = v0; v0 = v1; v1 = t; }
    out[0] = v0; out[1] = v1;
}

inline int edge_between(int va, int vb) {
    for (int e = 0; e < 12; ++e) {
        int ev[2];
        edge_endpoints(e, ev);
        if ((ev[0] == va && ev[1] == vb) || (ev[0] == vb && ev[1] == va)) return e;
    }
    return -1;
}

inline void build(Tables& T) {
    memset(&T, 0, sizeof(T));
    for (int e = 0; e < 12; ++e) edge_endpoints(e, T.edge_v[e]);
    for (int c = 0; c < 256; ++c) {
        for (int k = 0; k < 16; ++k) T.tri_edges[c][k] = -1;
        int neg[8];
        for (int v = 0; v < 8; ++v) neg[v] = (c >> v) & 1;
        // segments between crossed edges on every face
        int seg[24][2], nseg = 0;
        for (int a = 0; a < 3; ++a) {
            int b0 = (a == 0) ? 1 : 0, b1 = (a == 2) ? 1 : 2;
            for (int s = 0; s < 2; ++s) {
                static const int cu[4] = {0, 1, 1, 0}, cw[4] = {0, 0, 1, 1};
                int corner[4];
                for (int k = 0; k < 4; ++k) {
                    int p[3];
                    p[a] = s; p[b0] = cu[k]; p[b1] = cw[k];
                    corner[k] = vertex_id(p[0], p[1], p[2]);
                }
                int fe[4], cross[4], nc = 0;
                for (int k = 0; k < 4; ++k) {
                    fe[k] = edge_between(corner[k], corner[(k + 1) & 3]);
                    if (neg[corner[k]] != neg[corner[(k + 1) & 3]]) cross[nc++] = k;
                }
                if (nc == 2) {
                    seg[nseg][0] = fe[cross[0]]; seg[nseg][1] = fe[cross[1]]; ++nseg;
                } else if (nc == 4) {
                    if (neg[corner[0]]) {  // cut off corners 0 and 2
                        seg[nseg][0] = fe[3]; seg[nseg][1] = fe[0]; ++nseg;
                        seg[nseg][0] = fe[1]; seg[nseg][1] = fe[2]; ++nseg;
                    } else {               // cut off corners 1 and 3
                        seg[nseg][0] = fe[0]; seg[nseg][1] = fe[1]; ++nseg;
                        seg[nseg][0] = fe[2]; seg[nseg][1] = fe[3]; ++nseg;
                    }
                }
            }
        }
        // link segments into closed loops
        int used[24] = {0};
        int ntri = 0;
        for (int s0 = 0; s0 < nseg; ++s0) {
            if (used[s0]) continue;
            int loop[12], n = 0;
            used[s0] = 1;
            loop[n++] = seg[s0][0];
            int cur = seg[s0][1];
            while (cur != loop[0] && n < 12) {
                loop[n++] = cur;
                int nxt = -1;
                for (int s = 0; s < nseg; ++s) {
                    if (used[s]) continue;
                    if (seg[s][0] == cur) { nxt = seg[s][1]; used[s] = 1; break; }
                    if (seg[s][1] == cur) { nxt = seg[s][0]; used[s] = 1; break; }
                }
                if (nxt < 0) break;
                cur = nxt;
            }
            // orientation: Newell normal of the edge midpoints must point
            // away from the negative endpoint of each crossed edge
            double mid[12][3];
            for (int k = 0; k < n; ++k) {
                int p0[3], p1[3];
                vertex_xyz(T.edge_v[loop[k]][0], p0);
                vertex_xyz(T.edge_v[loop[k]][1], p1);
                for (int d = 0; d < 3; ++d) mid[k][d] = 0.5 * (p0[d] + p1[d]);
            }
            double nrm[3] = {0, 0, 0};
            for (int k = 0; k < n; ++k) {
                const double* u = mid[k];
                const double* w = mid[(k + 1) % n];
                nrm[0] += (u[1] - w[1]) * (u[2] + w[2]);
                nrm[1] += (u[2] - w[2]) * (u[0] + w[0]);
                nrm[2] += (u[0] - w[0]) * (u[1] + w[1]);
            }
            double dir = 0;
            for (int k = 0; k < n; ++k) {
                int ev0 = T.edge_v[loop[k]][0], ev1 = T.edge_v[loop[k]][1];
                int pin[3];
                vertex_xyz(neg[ev0] ? ev0 : ev1, pin);
                for (int d = 0; d < 3; ++d) dir += nrm[d] * (mid[k][d] - pin[d]);
            }
            if (dir < 0) {
                for (int k = 0; k < n / 2; ++k) {
                    int t = loop[k]; loop[k] = loop[n - 1 - k]; loop[n - 1 - k] = t;
                }
            }
            for (int k = 1; k + 1 < n; ++k) {
                T.tri_edges[c][3 * ntri + 0] = loop[0];
                T.tri_edges[c][3 * ntri + 1] = loop[k];
                T.tri_edges[c][3 * ntri + 2] = loop[k + 1];
                ++ntri;
            }
        }
        T.tri_count[c] = ntri;
    }
}

}  // namespace prgpu_mc
