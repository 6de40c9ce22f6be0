// Output writers in the reference's file formats: legacy VTK field files
// (src/IO_multiphase.cpp:500-714, VTK_legacy_writer_3D), the solid geometry
// VTK (:800-841, VTK_walls_bin) and the restart checkpoint (:252-305
// save_checkpoint, read back as src/Init_multiphase.cpp:501-537).
//
// The VTK bodies are assembled on the device: one thread per node derives
// the written quantities (the macroscopic variables of compute_macro_vars,
// src/Misc.cpp:222-274, for type 1) and stores them big-endian in the file's
// order, so only the finished body crosses to the host.  Built with
// -fmad=false: every derived value is the reference's IEEE expression in its
// order, and the files are byte-identical to the reference's for the same
// state.
#include <cstdio>
#include <string>
#include <vector>

#include "context.cuh"
#include "setup.cuh"

namespace mflbm {
namespace {

__device__ __forceinline__ void store_be(unsigned char* p, float v) {
    const unsigned int u = __float_as_uint(v);
    p[0] = (unsigned char)(u >> 24); p[1] = (unsigned char)(u >> 16);
    p[2] = (unsigned char)(u >> 8); p[3] = (unsigned char)u;
}
__device__ __forceinline__ void store_be(unsigned char* p, double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
#pragma unroll
    for (int b = 0; b < 8; ++b) p[b] = (unsigned char)(u >> (56 - 8 * b));
}
__device__ __forceinline__ void store_be(unsigned char* p, int v) { store_be(p, __int_as_float(v)); }

template <class T, class E> struct VtkArgs {
    Grid g;
    PopView<T, E> P;
    const void *phi, *cnx, *cny, *cnz, *cnorm, *curv;
    const int32_t* walls;
    double gamma, force_z;  // exact T values
    unsigned char* out;
};

// vtk_type 1: phi (0 on solids), density, velocity_X/Y/Z from post-even
// populations (compute_macro_vars); vtk_type 3: phi, c_norm, cn_x/y/z;
// vtk_type 2: phi (0 on solids) as float.  Five (or one) blocks of n0 values,
// node (i, j, k) at (i-1) + nx ((j-1) + ny (k-1)).
template <class T, class E, int TYPE>
__global__ void vtk_body_kernel(VtkArgs<T, E> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1, k = blockIdx.z + 1;
    const Grid& g = a.g;
    if (i > g.nx) return;
    const ll n0 = g.n0();
    const ll idx = (i - 1) + (ll)g.nx * ((j - 1) + (ll)g.ny * (k - 1));
    const T* phi = (const T*)a.phi;
    const int wall = a.walls[g.s2(i, j, k)];
    const T ph = phi[g.s4(i, j, k)];
    if (TYPE == 2) {
        const T p0 = T(0) * T(wall) + ph * T(1 - wall);
        store_be(a.out + 4 * idx, (float)p0);
        return;
    }
    unsigned char* o = a.out + sizeof(T) * idx;
    const ll blk = sizeof(T) * n0;
    if (TYPE == 3) {
        const ll n2 = g.s2(i, j, k);
        store_be(o, ph);
        store_be(o + blk, ((const T*)a.cnorm)[n2]);
        store_be(o + 2 * blk, ((const T*)a.cnx)[n2]);
        store_be(o + 3 * blk, ((const T*)a.cny)[n2]);
        store_be(o + 4 * blk, ((const T*)a.cnz)[n2]);
        return;
    }
    T f[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = a.P.get(i, j, k, q, 0) + a.P.get(i, j, k, q, 1);
    const T keep = T(1 - wall);
    T s = f[0];
#pragma unroll
    for (int q = 1; q < 19; ++q) s = s + f[q];
    const T rho = s * keep;
    const ll n2 = g.s2(i, j, k);
    const T tmp = T(0.5) * T(a.gamma) * ((const T*)a.curv)[g.s1(i, j, k)] * ((const T*)a.cnorm)[n2];
    const T fx = tmp * ((const T*)a.cnx)[n2];
    const T fy = tmp * ((const T*)a.cny)[n2];
    const T fz = tmp * ((const T*)a.cnz)[n2] + T(a.force_z);
    const T u = (f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14] - T(0.5) * fx) * keep;
    const T v = (f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18] - T(0.5) * fy) * keep;
    const T w = (f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18] - T(0.5) * fz) * keep;
    const T p0 = T(0) * T(wall) + ph * keep;
    store_be(o, p0);
    store_be(o + blk, rho);
    store_be(o + 2 * blk, u);
    store_be(o + 3 * blk, v);
    store_be(o + 4 * blk, w);
}

__global__ void walls_body_kernel(Grid g, const int32_t* walls, unsigned char* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y + 1, k = blockIdx.z + 1;
    if (i > g.nx) return;
    const ll idx = (i - 1) + (ll)g.nx * ((j - 1) + (ll)g.ny * (k - 1));
    store_be(out + 4 * idx, (int)walls[g.s2(i, j, k)]);
}

std::string vtk_header(const Grid& g, int ny_out, int nz_out) {
    char buf[512];
    snprintf(buf, sizeof buf,
             "# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET STRUCTURED_POINTS\nDIMENSIONS %d %d %d\n"
             "ORIGIN 1 1 1\nSPACING 1 1 1\nPOINT_DATA %lld\n",
             g.nx, ny_out, nz_out, (long long)g.nx * ny_out * nz_out);
    return buf;
}

int write_file(const char* path, const std::vector<std::pair<std::string, std::pair<const unsigned char*, size_t>>>& parts,
               const std::string& head) {
    FILE* f = fopen(path, "wb");
    if (!f) return fail(MFLBM_E_ARG, std::string("cannot create ") + path);
    bool ok = fwrite(head.data(), 1, head.size(), f) == head.size();
    for (const auto& p : parts) {
        ok = ok && fwrite(p.first.data(), 1, p.first.size(), f) == p.first.size();
        ok = ok && fwrite(p.second.first, 1, p.second.second, f) == p.second.second;
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? MFLBM_OK : fail(MFLBM_E_ARG, std::string("write failed: ") + path);
}

template <class T, class E>
int write_vtk_t(mflbm_context& c, int vtk_type, int precision_cmd, const char* path) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    const ll n0 = g.n0();
    const int nblk = vtk_type == 2 ? 1 : 5;
    const size_t vsize = vtk_type == 2 ? 4 : sizeof(T);
    const size_t bytes = (size_t)nblk * n0 * vsize;
    unsigned char* dout = (unsigned char*)d.staging;  // the population staging buffer holds 38 n1 values
    VtkArgs<T, E> a;
    a.g = g;
    a.P.p = (E*)d.pdf;
    a.P.b = d.b;
    a.phi = d.phi; a.cnx = d.cn_x; a.cny = d.cn_y; a.cnz = d.cn_z; a.cnorm = d.c_norm; a.curv = d.curv;
    a.walls = d.walls;
    a.gamma = (double)T(c.params.lbm_gamma);
    a.force_z = (double)T(c.params.force_z);
    a.out = dout;
    const dim3 grid(grid_for(g.nx, 128), g.ny, g.nz);
    if (vtk_type == 1) vtk_body_kernel<T, E, 1><<<grid, 128, 0, c.stream>>>(a);
    else if (vtk_type == 2) vtk_body_kernel<T, E, 2><<<grid, 128, 0, c.stream>>>(a);
    else vtk_body_kernel<T, E, 3><<<grid, 128, 0, c.stream>>>(a);
    int rc = after_launch("vtk_body");
    if (rc != MFLBM_OK) return rc;
    std::vector<unsigned char> host(bytes);
    MFLBM_CUDA(cudaMemcpyAsync(host.data(), dout, bytes, cudaMemcpyDeviceToHost, c.stream));
    MFLBM_CUDA(cudaStreamSynchronize(c.stream));
    // the type 1 / 3 files name the precision from output_fieldData_precision_cmd
    // but hold values of the solver precision (src/IO_multiphase.cpp:611-620)
    const std::string fmt = vtk_type == 2 ? "float" : (precision_cmd == 0 ? "float" : "double");
    static const char* names[5] = {"phi", "density", "velocity_X", "velocity_Y", "velocity_Z"};
    std::vector<std::pair<std::string, std::pair<const unsigned char*, size_t>>> parts;
    for (int b = 0; b < nblk; ++b)
        parts.push_back({std::string("SCALARS ") + names[b] + " " + fmt + "\nLOOKUP_TABLE default\n",
                         {host.data() + (size_t)b * n0 * vsize, (size_t)n0 * vsize}});
    return write_file(path, parts, vtk_header(g, g.ny, g.nz));
}

template <class T>
int write_checkpoint_t(mflbm_context& c, int ntime, const char* path) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    int rc = convert_populations(c, false);
    if (rc != MFLBM_OK) return rc;
    std::vector<T> pdf((size_t)g.n1() * 38), phi((size_t)g.n4());
    MFLBM_CUDA(cudaMemcpyAsync(pdf.data(), d.staging, sizeof(T) * pdf.size(), cudaMemcpyDeviceToHost, c.stream));
    MFLBM_CUDA(cudaMemcpyAsync(phi.data(), d.phi, sizeof(T) * phi.size(), cudaMemcpyDeviceToHost, c.stream));
    const size_t pl = (size_t)g.plane1();
    std::vector<T> fcv, gcv, pcv;
    if (c.params.outlet_BC == 1) {
        fcv.resize(pl * 19); gcv.resize(pl * 19); pcv.resize(pl);
        MFLBM_CUDA(cudaMemcpyAsync(fcv.data(), d.f_cv, sizeof(T) * fcv.size(), cudaMemcpyDeviceToHost, c.stream));
        MFLBM_CUDA(cudaMemcpyAsync(gcv.data(), d.g_cv, sizeof(T) * gcv.size(), cudaMemcpyDeviceToHost, c.stream));
        MFLBM_CUDA(cudaMemcpyAsync(pcv.data(), d.phi_cv, sizeof(T) * pcv.size(), cudaMemcpyDeviceToHost, c.stream));
    }
    MFLBM_CUDA(cudaStreamSynchronize(c.stream));
    FILE* f = fopen(path, "wb");
    if (!f) return fail(MFLBM_E_ARG, std::string("cannot create ") + path);
    const int nt_next = ntime + 1;
    const T fz = T(c.params.force_z), rin = T(c.params.rho_in);
    bool ok = fwrite(&nt_next, sizeof(int), 1, f) == 1 && fwrite(&fz, sizeof(T), 1, f) == 1 &&
              fwrite(&rin, sizeof(T), 1, f) == 1 && fwrite(pdf.data(), sizeof(T), pdf.size(), f) == pdf.size() &&
              fwrite(phi.data(), sizeof(T), phi.size(), f) == phi.size();
    if (c.params.outlet_BC == 1)
        ok = ok && fwrite(fcv.data(), sizeof(T), fcv.size(), f) == fcv.size() &&
             fwrite(gcv.data(), sizeof(T), gcv.size(), f) == gcv.size() &&
             fwrite(pcv.data(), sizeof(T), pcv.size(), f) == pcv.size();
    ok = (fclose(f) == 0) && ok;
    return ok ? MFLBM_OK : fail(MFLBM_E_ARG, std::string("write failed: ") + path);
}

}  // namespace

int write_vtk(mflbm_context& c, int vtk_type, int precision_cmd, const char* path) {
    if (c.params.precision == MFLBM_FP64) return write_vtk_t<double, double>(c, vtk_type, precision_cmd, path);
    if (c.params.storage == MFLBM_STORE_F16) return write_vtk_t<float, __half>(c, vtk_type, precision_cmd, path);
    if (c.params.storage == MFLBM_STORE_BF16) return write_vtk_t<float, __nv_bfloat16>(c, vtk_type, precision_cmd, path);
    return write_vtk_t<float, float>(c, vtk_type, precision_cmd, path);
}

int write_walls_vtk(mflbm_context& c, const char* path) {
    DeviceState& d = c.d;
    const Grid g = d.g;
    const size_t bytes = (size_t)4 * g.n0();
    unsigned char* dout = (unsigned char*)d.staging;
    walls_body_kernel<<<dim3(grid_for(g.nx, 128), g.ny, g.nz), 128, 0, c.stream>>>(g, d.walls, dout);
    int rc = after_launch("walls_body");
    if (rc != MFLBM_OK) return rc;
    std::vector<unsigned char> host(bytes);
    MFLBM_CUDA(cudaMemcpyAsync(host.data(), dout, bytes, cudaMemcpyDeviceToHost, c.stream));
    MFLBM_CUDA(cudaStreamSynchronize(c.stream));
    return write_file(path, {{"SCALARS walls int\nLOOKUP_TABLE default\n", {host.data(), bytes}}},
                      vtk_header(g, g.ny, g.nz));
}

int write_checkpoint(mflbm_context& c, int ntime, const char* path) {
    return c.params.precision == MFLBM_FP32 ? write_checkpoint_t<float>(c, ntime, path)
                                            : write_checkpoint_t<double>(c, ntime, path);
}

}  // namespace mflbm
