// Mass properties of many meshes on the device: the reference's mesh set-up
// (model/mesh.cpp:53-91 initInertiaDataVolume, :93-130
// initInertiaDataSurface; model/inertia.cpp:20-84) for large mesh sets, such
// as the 16,384 distinct noisy icospheres of the open-box scene.
//
// In the operation order of the library's host set-up (host/d2g_scene.cpp
// mass_volume / mass_surface), so a mesh gets the same bits on the GPU as on
// the host:
//   * closed surfaces (volume model): the tetrahedra of the faces with the
//     origin (the reference tetrahedralises with tetgen, absent here; the sum
//     over face tetrahedra is the divergence theorem's exact volume
//     integral): volume, centre of mass, then the unit-density inertia tensor
//     about the centre of mass with tetrahedronInertiaTensor's terms;
//   * thin shells (surface model): triangle area times thickness per face,
//     the centroid-weighted centre of mass, then the point inertia tensors of
//     the three vertices per face;
//   * the inverse of the 3x3 tensor by cofactors.
// One warp per mesh: the lanes compute the terms of 32 faces at a time into
// shared memory, then lane k adds accumulator k's terms face by face, so
// every sum is the same left-to-right chain as on the host (bit-identical)
// while the per-face arithmetic, nearly all of the FP64 work, runs 32 wide.
#include "d2g_geom.cuh"
#include "d2g_internal.hpp"

namespace d2g {
namespace {

constexpr int kMassWarps = 4;    // meshes per block
constexpr int kMassStride = 29;  // terms per face slot (at most 27), odd: no bank conflicts

__device__ V3 mvert(const double* V, const int32_t* F, int f, int k) {
    const double* p = V + 3 * (size_t)F[3 * (size_t)f + k];
    return mk(p[0], p[1], p[2]);
}

// model/inertia.cpp:20-73 tetrahedronInertiaTensor (Tonon 2005) with the
// reference's placement of the product terms; `sign` carries the orientation.
// Writes the tetrahedron's 9 tensor entries (row major) to R.
__device__ void tet_inertia_terms(V3 a, V3 b, V3 c, V3 d, double sign, double* R) {
    const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z}, C[3] = {c.x, c.y, c.z}, D[3] = {d.x, d.y, d.z};
    const double detJ = dot(a - d, cross(b - d, c - d));
    auto sq = [&](int k) {
        return A[k] * A[k] + A[k] * B[k] + B[k] * B[k] + A[k] * C[k] + B[k] * C[k] + C[k] * C[k] + A[k] * D[k] +
               B[k] * D[k] + C[k] * D[k] + D[k] * D[k];
    };
    auto pr = [&](int i, int j) {
        return 2 * A[i] * A[j] + B[i] * A[j] + C[i] * A[j] + D[i] * A[j] + A[i] * B[j] + 2 * B[i] * B[j] +
               C[i] * B[j] + D[i] * B[j] + A[i] * C[j] + B[i] * C[j] + 2 * C[i] * C[j] + D[i] * C[j] + A[i] * D[j] +
               B[i] * D[j] + C[i] * D[j] + 2 * D[i] * D[j];
    };
    const double ixx = sign * detJ * (sq(1) + sq(2)) / 60;
    const double iyy = sign * detJ * (sq(0) + sq(2)) / 60;
    const double izz = sign * detJ * (sq(0) + sq(1)) / 60;
    const double iyz = -sign * detJ * pr(1, 2) / 120;
    const double ixy = -sign * detJ * pr(0, 2) / 120;
    const double ixz = -sign * detJ * pr(0, 1) / 120;
    R[0] = ixx;
    R[1] = ixy;
    R[2] = ixz;
    R[3] = ixy;
    R[4] = iyy;
    R[5] = iyz;
    R[6] = ixz;
    R[7] = iyz;
    R[8] = izz;
}

__device__ void inv3_cofactor(const double* m, double* r) {
    const double c00 = m[4] * m[8] - m[5] * m[7];
    const double c01 = m[5] * m[6] - m[3] * m[8];
    const double c02 = m[3] * m[7] - m[4] * m[6];
    const double det = (m[0] * c00 + m[1] * c01) + m[2] * c02;
    const double id = 1.0 / det;
    r[0] = c00 * id;
    r[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    r[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    r[3] = c01 * id;
    r[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    r[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    r[6] = c02 * id;
    r[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    r[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

__device__ double area3(V3 A, V3 B, V3 C) { return 0.5 * norm(cross(A - C, B - C)); }

// Adds the terms the warp's lanes wrote for faces [0, cnt) of a chunk to the
// accumulator of this lane (lane < nacc), in face order; a face holds `per`
// terms per accumulator, added in turn.
__device__ double chain_add(double acc, const double (*T)[kMassStride], int cnt, int lane, int nacc, int per) {
    if (lane < nacc)
        for (int j = 0; j < cnt; j++)
            for (int k = 0; k < per; k++) acc += T[j][per * lane + k];
    __syncwarp();
    return acc;
}

// out per mesh (22 doubles): volume, centre of mass (3), unit-density inertia
// tensor about it (9, row major), its inverse (9).
__global__ void __launch_bounds__(32 * kMassWarps) k_mass_props(int n, const double* __restrict__ V,
                                                                const int32_t* __restrict__ F,
                                                                const int32_t* __restrict__ voff,
                                                                const int32_t* __restrict__ foff,
                                                                const uint8_t* __restrict__ surface, double thickness,
                                                                double* __restrict__ out) {
    __shared__ double terms[kMassWarps][32][kMassStride];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m = blockIdx.x * kMassWarps + warp;
    if (m >= n) return;  // whole warps leave together
    double(*T)[kMassStride] = terms[warp];
    const double* Vm = V + 3 * (size_t)voff[m];
    const int f0 = foff[m], f1 = foff[m + 1];
    const bool shell = surface && surface[m];

    // pass 1: lane 0 sums the volume, lanes 1..3 the centre of mass
    double acc = 0.0;
    for (int base = f0; base < f1; base += 32) {
        const int f = base + lane, cnt = min(32, f1 - base);
        if (f < f1) {
            double* t = T[lane];
            const V3 a = mvert(Vm, F, f, 0), b = mvert(Vm, F, f, 1), c = mvert(Vm, F, f, 2);
            if (shell) {
                const double tv = area3(a, b, c) * thickness;
                const V3 w = (((a + b) + c) * (1.0 / 3.0)) * tv;
                t[0] = tv;
                t[1] = w.x;
                t[2] = w.y;
                t[3] = w.z;
            } else {
                const double v = dot(a, cross(b, c)) / 6.0;
                const V3 w = ((a + b) + c) * (v / 4.0);
                t[0] = v;
                t[1] = w.x;
                t[2] = w.y;
                t[3] = w.z;
            }
        }
        __syncwarp();
        acc = chain_add(acc, T, cnt, lane, 4, 1);
    }
    const double vol = __shfl_sync(0xffffffffu, acc, 0);
    const double inv_vol = 1.0 / vol;
    const V3 com = mk(__shfl_sync(0xffffffffu, acc, 1) * inv_vol, __shfl_sync(0xffffffffu, acc, 2) * inv_vol,
                      __shfl_sync(0xffffffffu, acc, 3) * inv_vol);

    // pass 2: lane k < 9 sums entry k of the inertia tensor about the centre of mass
    acc = 0.0;
    for (int base = f0; base < f1; base += 32) {
        const int f = base + lane, cnt = min(32, f1 - base);
        if (f < f1) {
            double* t = T[lane];
            const V3 A = mvert(Vm, F, f, 0) - com, B = mvert(Vm, F, f, 1) - com, C = mvert(Vm, F, f, 2) - com;
            if (shell) {
                const double tv = area3(A, B, C) * thickness;
                const V3 P[3] = {A, B, C};
                for (int k = 0; k < 3; k++) {  // model/inertia.cpp:75-84 pointInertiaTensor
                    const double x = P[k].x, y = P[k].y, z = P[k].z;
                    const double pi[9] = {y * y + z * z, -x * y, -x * z, -x * y, x * x + z * z, -y * z,
                                          -x * z, -y * z, x * x + y * y};
                    for (int j = 0; j < 9; j++) t[3 * j + k] = tv * pi[j] / 3.0;
                }
            } else {
                tet_inertia_terms(A, B, C, mk(0, 0, 0), 1.0, t);
            }
        }
        __syncwarp();
        acc = chain_add(acc, T, cnt, lane, 9, shell ? 3 : 1);
    }
    double I[9], Ii[9];
    for (int k = 0; k < 9; k++) I[k] = __shfl_sync(0xffffffffu, acc, k);
    if (lane == 0) {
        inv3_cofactor(I, Ii);
        double* o = out + 22 * (size_t)m;
        o[0] = vol;
        o[1] = com.x;
        o[2] = com.y;
        o[3] = com.z;
        for (int k = 0; k < 9; k++) {
            o[4 + k] = I[k];
            o[13 + k] = Ii[k];
        }
    }
}

}  // namespace

int run_mass_properties(d2g_ctx* ctx, const double* d_V, const int32_t* d_F, const int32_t* d_voff,
                        const int32_t* d_foff, const uint8_t* d_surface, int n_meshes, double thickness,
                        double* d_out) {
    if (n_meshes > 0) {
        k_mass_props<<<(n_meshes + kMassWarps - 1) / kMassWarps, 32 * kMassWarps, 0, ctx->stream>>>(
            n_meshes, d_V, d_F, d_voff, d_foff, d_surface, thickness, d_out);
        ctx->eng.launches++;
    }
    D2G_CUDA(cudaGetLastError());
    return D2G_OK;
}

}  // namespace d2g
