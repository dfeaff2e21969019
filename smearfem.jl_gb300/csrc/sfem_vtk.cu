// VTK output of the reference's post-processing (src/PostProcess.jl:258-304):
//   sfem_vtk_write        write_vtk:   one UnstructuredGrid (.vtu) with one
//                                      point field
//   sfem_vtk_write_scene  write_scene: one .vtu per step plus a ParaView
//                                      collection (.pvd), step i at time i-1
// Files are VTK XML with the arrays in an appended raw block (UInt64 byte
// counts, little-endian), which ParaView and the VTK readers take as they
// are.  Points are written with three components (2D meshes get z = 0),
// connectivity 0-based, cells by element size (8: hexahedron, 4: quad,
// 2: line).  Host input needs no GPU.  Device input is copied to the host
// through two pinned buffers, so that while one step is written to disk the
// next one is already on its way from the GPU.
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "sfem_internal.cuh"

namespace {

struct Out {
    FILE *f = nullptr;
    bool ok = true;
    void raw(const void *p, size_t n) {
        if (ok && n && fwrite(p, 1, n, f) != n) ok = false;
    }
    void str(const std::string &s) { raw(s.data(), s.size()); }
};

int vtk_cell_type(int nen) { return nen == 8 ? 12 : nen == 4 ? 9 : nen == 2 ? 3 : -1; }

// One .vtu; X, ien, field are host arrays in the reference's layouts.
int write_vtu(sfem_ctx *ctx, const std::string &path, const double *X, int ndim, int64_t nN, const int64_t *ien,
              int64_t nEl, int nen, const char *name, const double *field, int ncomp) {
    Out o;
    o.f = fopen(path.c_str(), "wb");
    if (!o.f) return ctx ? sfem_set_error(ctx, SFEM_BAD_ARG, "cannot open %s for writing", path.c_str()) : SFEM_BAD_ARG;
    const uint64_t bpts = sizeof(double) * 3 * nN, bcon = sizeof(int64_t) * nen * nEl, boff = sizeof(int64_t) * nEl,
                   btyp = (uint64_t)nEl, bfld = field ? sizeof(double) * ncomp * nN : 0;
    uint64_t off = 0;
    char buf[512];
    o.str("<?xml version=\"1.0\"?>\n"
          "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
          "  <UnstructuredGrid>\n");
    snprintf(buf, sizeof(buf), "    <Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", (long long)nN,
             (long long)nEl);
    o.str(buf);
    o.str("      <Points>\n");
    snprintf(buf, sizeof(buf),
             "        <DataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\" format=\"appended\" "
             "offset=\"%llu\"/>\n",
             (unsigned long long)off);
    o.str(buf);
    off += 8 + bpts;
    o.str("      </Points>\n      <Cells>\n");
    snprintf(buf, sizeof(buf),
             "        <DataArray type=\"Int64\" Name=\"connectivity\" format=\"appended\" offset=\"%llu\"/>\n",
             (unsigned long long)off);
    o.str(buf);
    off += 8 + bcon;
    snprintf(buf, sizeof(buf),
             "        <DataArray type=\"Int64\" Name=\"offsets\" format=\"appended\" offset=\"%llu\"/>\n",
             (unsigned long long)off);
    o.str(buf);
    off += 8 + boff;
    snprintf(buf, sizeof(buf),
             "        <DataArray type=\"UInt8\" Name=\"types\" format=\"appended\" offset=\"%llu\"/>\n",
             (unsigned long long)off);
    o.str(buf);
    off += 8 + btyp;
    o.str("      </Cells>\n");
    if (field) {
        snprintf(buf, sizeof(buf),
                 "      <PointData>\n        <DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"%d\" "
                 "format=\"appended\" offset=\"%llu\"/>\n      </PointData>\n",
                 name, ncomp, (unsigned long long)off);
        o.str(buf);
    }
    o.str("    </Piece>\n  </UnstructuredGrid>\n  <AppendedData encoding=\"raw\">\n_");
    // points, padded to 3 components
    o.raw(&bpts, 8);
    {
        std::vector<double> chunk;
        const int64_t step = 1 << 16;
        for (int64_t m0 = 0; m0 < nN; m0 += step) {
            const int64_t m1 = m0 + step < nN ? m0 + step : nN;
            chunk.assign((size_t)(3 * (m1 - m0)), 0.0);
            for (int64_t m = m0; m < m1; ++m)
                for (int k = 0; k < ndim && k < 3; ++k) chunk[(m - m0) * 3 + k] = X[m * ndim + k];
            o.raw(chunk.data(), chunk.size() * sizeof(double));
        }
    }
    // cells: IEN is nEl x nen, column-major, 1-based
    o.raw(&bcon, 8);
    {
        std::vector<int64_t> chunk;
        const int64_t step = 1 << 14;
        for (int64_t e0 = 0; e0 < nEl; e0 += step) {
            const int64_t e1 = e0 + step < nEl ? e0 + step : nEl;
            chunk.resize((size_t)(nen * (e1 - e0)));
            for (int64_t e = e0; e < e1; ++e)
                for (int a = 0; a < nen; ++a) chunk[(e - e0) * nen + a] = ien[e + a * nEl] - 1;
            o.raw(chunk.data(), chunk.size() * sizeof(int64_t));
        }
    }
    o.raw(&boff, 8);
    {
        std::vector<int64_t> offs((size_t)nEl);
        for (int64_t e = 0; e < nEl; ++e) offs[e] = (e + 1) * nen;
        o.raw(offs.data(), offs.size() * sizeof(int64_t));
    }
    o.raw(&btyp, 8);
    {
        std::vector<uint8_t> types((size_t)nEl, (uint8_t)vtk_cell_type(nen));
        o.raw(types.data(), types.size());
    }
    if (field) {
        o.raw(&bfld, 8);
        o.raw(field, bfld);  // ncomp x nN column-major = point-major components
    }
    o.str("\n  </AppendedData>\n</VTKFile>\n");
    const bool closed = fclose(o.f) == 0;
    if (!o.ok || !closed)
        return ctx ? sfem_set_error(ctx, SFEM_BAD_ARG, "writing %s failed", path.c_str()) : SFEM_BAD_ARG;
    return SFEM_OK;
}

// Host copies of the mesh arrays (device input is copied once).
struct HostMesh {
    std::vector<double> X;
    std::vector<int64_t> ien;
    const double *x = nullptr;
    const int64_t *e = nullptr;
};

int host_mesh(sfem_ctx *ctx, const double *NodeList, int ndim, int64_t nN, const int64_t *IEN, int64_t nEl, int nen,
              int mem_space, HostMesh &h) {
    if (mem_space == SFEM_MEM_HOST) {
        h.x = NodeList;
        h.e = IEN;
        return SFEM_OK;
    }
    h.X.resize((size_t)(ndim * nN));
    h.ien.resize((size_t)(nen * nEl));
    SFEM_CUDA(ctx, cudaMemcpy(h.X.data(), NodeList, sizeof(double) * ndim * nN, cudaMemcpyDeviceToHost));
    SFEM_CUDA(ctx, cudaMemcpy(h.ien.data(), IEN, sizeof(int64_t) * nen * nEl, cudaMemcpyDeviceToHost));
    h.x = h.X.data();
    h.e = h.ien.data();
    return SFEM_OK;
}

int check_args(sfem_ctx *ctx, const char *path, const double *NodeList, int ndim, int64_t nN, const int64_t *IEN,
               int64_t nEl, int nen, int ncomp, int mem_space) {
    if (!path || !NodeList || nN < 1 || (nEl > 0 && !IEN) || nEl < 0 || ndim < 1 || ndim > 3 ||
        vtk_cell_type(nen) < 0 || ncomp < 1)
        return ctx ? sfem_set_error(ctx, SFEM_BAD_ARG, "bad VTK arguments") : SFEM_BAD_ARG;
    if (mem_space != SFEM_MEM_HOST && mem_space != SFEM_MEM_DEVICE) return SFEM_BAD_ARG;
    if (mem_space == SFEM_MEM_DEVICE && !ctx) return SFEM_BAD_ARG;
    return SFEM_OK;
}

}  // namespace

extern "C" int sfem_vtk_write(sfem_ctx *ctx, const char *path, const double *NodeList, int ndim, int64_t nNodes,
                              const int64_t *IEN, int64_t nEl, int nen, const char *field_name, const double *field,
                              int ncomp, int mem_space) {
    SFEM_TRY(check_args(ctx, path, NodeList, ndim, nNodes, IEN, nEl, nen, ncomp, mem_space));
    HostMesh h;
    if (mem_space == SFEM_MEM_DEVICE) cudaSetDevice(ctx->device);
    SFEM_TRY(host_mesh(ctx, NodeList, ndim, nNodes, IEN, nEl, nen, mem_space, h));
    std::vector<double> hf;
    const double *fp = field;
    if (field && mem_space == SFEM_MEM_DEVICE) {
        hf.resize((size_t)(ncomp * nNodes));
        SFEM_CUDA(ctx, cudaMemcpy(hf.data(), field, sizeof(double) * ncomp * nNodes, cudaMemcpyDeviceToHost));
        fp = hf.data();
    }
    return write_vtu(ctx, path, h.x, ndim, nNodes, h.e, nEl, nen, field_name ? field_name : "u", fp, ncomp);
}

extern "C" int sfem_vtk_write_scene(sfem_ctx *ctx, const char *basename, const double *NodeList, int ndim,
                                    int64_t nNodes, const int64_t *IEN, int64_t nEl, int nen, const double *fields,
                                    int ncomp, int64_t nsteps, int mem_space) {
    SFEM_TRY(check_args(ctx, basename, NodeList, ndim, nNodes, IEN, nEl, nen, ncomp, mem_space));
    if (nsteps < 0 || (nsteps > 0 && !fields)) return ctx ? sfem_set_error(ctx, SFEM_BAD_ARG, "bad fields") : SFEM_BAD_ARG;
    const bool dev = mem_space == SFEM_MEM_DEVICE;
    if (dev) cudaSetDevice(ctx->device);
    HostMesh h;
    SFEM_TRY(host_mesh(ctx, NodeList, ndim, nNodes, IEN, nEl, nen, mem_space, h));
    const std::string base(basename);
    // file names of WriteVTK's vtk_grid(string(fileName, "timestep_$i")) and
    // paraview_collection(string(fileName, "displacement"))
    const size_t slash = base.find_last_of('/');
    const std::string stem = slash == std::string::npos ? base : base.substr(slash + 1);
    const size_t per = (size_t)ncomp * (size_t)nNodes;
    double *pinned[2] = {nullptr, nullptr};
    cudaEvent_t ready[2] = {nullptr, nullptr};
    int st = SFEM_OK;
    if (dev) {
        for (int k = 0; k < 2 && st == SFEM_OK; ++k) {
            st = sfem_cuda_status(ctx, cudaMallocHost((void **)&pinned[k], sizeof(double) * (per ? per : 1)),
                                  "pinned VTK buffer");
            if (st == SFEM_OK) st = sfem_cuda_status(ctx, cudaEventCreateWithFlags(&ready[k], cudaEventDisableTiming),
                                                     "event");
        }
        if (st == SFEM_OK && nsteps > 0) {
            st = sfem_cuda_status(ctx, cudaMemcpyAsync(pinned[0], fields, sizeof(double) * per, cudaMemcpyDeviceToHost,
                                                       ctx->stream), "D2H");
            if (st == SFEM_OK) st = sfem_cuda_status(ctx, cudaEventRecord(ready[0], ctx->stream), "event");
        }
    }
    std::string pvd = "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"1.0\" "
                      "byte_order=\"LittleEndian\" header_type=\"UInt64\">\n  <Collection>\n";
    for (int64_t i = 0; i < nsteps && st == SFEM_OK; ++i) {
        const double *fp = fields + (size_t)i * per;
        if (dev) {
            if (i + 1 < nsteps) {  // next step's copy runs while this one is written
                st = sfem_cuda_status(ctx, cudaMemcpyAsync(pinned[(i + 1) & 1], fields + (size_t)(i + 1) * per,
                                                           sizeof(double) * per, cudaMemcpyDeviceToHost, ctx->stream),
                                      "D2H");
                if (st == SFEM_OK) st = sfem_cuda_status(ctx, cudaEventRecord(ready[(i + 1) & 1], ctx->stream), "event");
                if (st != SFEM_OK) break;
            }
            if ((st = sfem_cuda_status(ctx, cudaEventSynchronize(ready[i & 1]), "D2H wait"))) break;
            fp = pinned[i & 1];
        }
        const std::string name = base + "timestep_" + std::to_string(i + 1) + ".vtu";
        // buffer i&1 is reused for step i+2 only after this synchronous write returns
        st = write_vtu(ctx, name, h.x, ndim, nNodes, h.e, nEl, nen, "u", fp, ncomp);
        char line[512];
        snprintf(line, sizeof(line), "    <DataSet timestep=\"%lld\" part=\"0\" file=\"%stimestep_%lld.vtu\"/>\n",
                 (long long)i, stem.c_str(), (long long)(i + 1));
        pvd += line;
    }
    if (dev) {
        cudaStreamSynchronize(ctx->stream);
        for (int k = 0; k < 2; ++k) {
            if (pinned[k]) cudaFreeHost(pinned[k]);
            if (ready[k]) cudaEventDestroy(ready[k]);
        }
    }
    if (st != SFEM_OK) return st;
    pvd += "  </Collection>\n</VTKFile>\n";
    const std::string pvd_path = base + "displacement.pvd";
    FILE *f = fopen(pvd_path.c_str(), "wb");
    if (!f) return ctx ? sfem_set_error(ctx, SFEM_BAD_ARG, "cannot open %s", pvd_path.c_str()) : SFEM_BAD_ARG;
    const bool ok = fwrite(pvd.data(), 1, pvd.size(), f) == pvd.size();
    if (fclose(f) != 0 || !ok) return ctx ? sfem_set_error(ctx, SFEM_BAD_ARG, "writing %s failed", pvd_path.c_str())
                                          : SFEM_BAD_ARG;
    return SFEM_OK;
}
