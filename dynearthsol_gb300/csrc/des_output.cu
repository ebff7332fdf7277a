// des_output.cu -- output frames in the reference's .save format
// (des_write_save_host, des_write_save).
//
// The layout is BinaryOutput's (binaryio.cxx:16-37): the file starts with a
// 4096-byte zero-padded ASCII header -- the revision line, then one
// "name<TAB>offset<LF>" line per array, offset being the array's first byte
// in the file -- and the arrays follow from byte 4096 on, in the order of
// Output::write (output.cxx:79-195).  The header is written last, over the
// reserved first 4096 bytes, as the arrays' offsets are known only then.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "des_ctx.cuh"
#include "des_kernels.cuh"

namespace {

constexpr size_t kHeaderLen = 4096;

struct SaveWriter {
    std::FILE *f = nullptr;
    std::string header;
    long eof = (long)kHeaderLen;
    bool ok = true;

    SaveWriter(const char *name, int ndims)
    {
        f = std::fopen(name, "wb");
        if (!f) {
            ok = false;
            return;
        }
        char line[64];
        std::snprintf(line, sizeof line, "# DynEarthSol ndims=%d revision=3\n", ndims);
        header = line;
        ok = std::fseek(f, eof, SEEK_SET) == 0;
    }

    void put(const char *name, const void *data, size_t elem, size_t count)
    {
        if (!ok) return;
        char line[256];
        const int len = std::snprintf(line, sizeof line, "%s\t%ld\n", name, eof);
        if (len <= 0 || (size_t)len >= sizeof line || header.size() + len >= kHeaderLen) {
            ok = false;   // the reference exits with 12 here (binaryio.cxx:85-94)
            return;
        }
        header += line;
        const size_t n = std::fwrite(data, elem, count, f);
        eof += (long)(n * elem);
        if (n != count) ok = false;
    }

    bool close()
    {
        if (!f) return false;
        std::vector<char> buf(kHeaderLen, 0);
        std::memcpy(buf.data(), header.data(), header.size());
        if (ok) ok = std::fseek(f, 0, SEEK_SET) == 0 && std::fwrite(buf.data(), 1, kHeaderLen, f) == kHeaderLen;
        ok = (std::fclose(f) == 0) && ok;
        f = nullptr;
        return ok;
    }
};

}  // namespace

int des_write_save_host(const char *filename, const des_save_frame *fr)
{
    if (!filename || !fr || (fr->ndims != 2 && fr->ndims != 3) || fr->nnode <= 0 || fr->nelem <= 0)
        return DES_EINPUT;
    const void *req[] = {fr->coord, fr->connectivity, fr->vel, fr->temperature, fr->plstrain, fr->delta_plstrain,
                         fr->strain_rate, fr->strain, fr->stress, fr->density, fr->mesh_quality, fr->viscosity,
                         fr->material, fr->force, fr->coord0, fr->bcflag};
    for (const void *q : req)
        if (!q) return DES_EINPUT;
    const size_t nd = fr->ndims, nn = fr->nnode, ne = fr->nelem, npe = nd + 1, nstr = nd * (nd + 1) / 2;
    const size_t D = sizeof(double);
    SaveWriter w(filename, fr->ndims);
    w.put("coordinate", fr->coord, D, nn * nd);
    w.put("connectivity", fr->connectivity, sizeof(int), ne * npe);
    w.put("velocity", fr->vel, D, nn * nd);
    w.put("temperature", fr->temperature, D, nn);
    w.put("plastic strain", fr->plstrain, D, ne);
    w.put("plastic strain-rate", fr->delta_plstrain, D, ne);
    w.put("strain-rate", fr->strain_rate, D, ne * nstr);
    w.put("strain", fr->strain, D, ne * nstr);
    w.put("stress", fr->stress, D, ne * nstr);
    w.put("density", fr->density, D, ne);
    w.put("mesh quality", fr->mesh_quality, D, ne);
    w.put("viscosity", fr->viscosity, D, ne);
    w.put("material", fr->material, D, ne);
    w.put("force", fr->force, D, nn * nd);
    w.put("coord0", fr->coord0, D, nn * nd);
    w.put("bcflag", fr->bcflag, sizeof(unsigned), nn);
    return w.close() ? DES_OK : DES_EINPUT;
}

using namespace des;

int des_write_save(des_ctx *c, const char *filename)
{
    if (!c || !filename) return DES_EINPUT;
    if (!c->has_state) return ctx_fail(c, DES_EINPUT, "des_write_save before des_upload_state");
    const KP &p = c->kp;
    const int nd = c->nd, nn = c->nn, ne = c->ne, npe = c->npe, nstr = c->nstr;
    double *d_out = nullptr;
    cudaError_t e = cudaMalloc((void **)&d_out, (size_t)4 * ne * sizeof(double));
    if (e != cudaSuccess) return ctx_cuda_fail(c, e, "cudaMalloc (output frame)");
    int rc = ctx_check_launch(c, launch_output_elem(p, d_out, c->stream));
    std::vector<double> coord((size_t)nn * nd), vel((size_t)nn * nd), T(nn), force((size_t)nn * nd),
        coord0((size_t)nn * nd), pls(ne), dpls(ne), srate((size_t)ne * nstr), strain((size_t)ne * nstr),
        stress((size_t)ne * nstr), ev((size_t)4 * ne);
    std::vector<int> conn((size_t)ne * npe), conn_soa((size_t)ne * npe);
    std::vector<unsigned> bc(nn);
    if (!rc) rc = ctx_get_field(c, p.x, coord.data(), nn, nd);
    if (!rc) rc = ctx_get_field(c, p.v, vel.data(), nn, nd);
    if (!rc) rc = ctx_get_field(c, p.T, T.data(), nn, 1);
    if (!rc) rc = ctx_get_field(c, p.pls, pls.data(), ne, 1);
    if (!rc) rc = ctx_get_field(c, p.dpls, dpls.data(), ne, 1);
    if (!rc) rc = ctx_get_field(c, p.srate, srate.data(), ne, nstr);
    if (!rc) rc = ctx_get_field(c, p.strain, strain.data(), ne, nstr);
    if (!rc) rc = ctx_get_field(c, p.stress, stress.data(), ne, nstr);
    if (!rc) rc = ctx_get_field(c, p.f, force.data(), nn, nd);
    if (!rc) rc = ctx_get_field(c, p.x0, coord0.data(), nn, nd);
    if (!rc && (e = cudaMemcpyAsync(ev.data(), d_out, ev.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                    c->stream)) != cudaSuccess)
        rc = ctx_cuda_fail(c, e, "cudaMemcpyAsync (output frame)");
    if (!rc && (e = cudaMemcpyAsync(conn_soa.data(), p.conn, conn_soa.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                    c->stream)) != cudaSuccess)
        rc = ctx_cuda_fail(c, e, "cudaMemcpyAsync (connectivity)");
    if (!rc && (e = cudaMemcpyAsync(bc.data(), p.bcflag, bc.size() * sizeof(unsigned), cudaMemcpyDeviceToHost,
                                    c->stream)) != cudaSuccess)
        rc = ctx_cuda_fail(c, e, "cudaMemcpyAsync (bcflag)");
    if (!rc && (e = cudaStreamSynchronize(c->stream)) != cudaSuccess) rc = ctx_cuda_fail(c, e, "cudaStreamSynchronize");
    cudaFree(d_out);
    if (rc) return rc;
    for (int i = 0; i < npe; ++i)
        for (int el = 0; el < ne; ++el) conn[(size_t)el * npe + i] = conn_soa[(size_t)i * ne + el];
    des_save_frame fr{};
    fr.ndims = nd;
    fr.nnode = nn;
    fr.nelem = ne;
    fr.coord = coord.data();
    fr.connectivity = conn.data();
    fr.vel = vel.data();
    fr.temperature = T.data();
    fr.plstrain = pls.data();
    fr.delta_plstrain = dpls.data();
    fr.strain_rate = srate.data();
    fr.strain = strain.data();
    fr.stress = stress.data();
    fr.density = ev.data();
    fr.mesh_quality = ev.data() + ne;
    fr.viscosity = ev.data() + 2 * (size_t)ne;
    fr.material = ev.data() + 3 * (size_t)ne;
    fr.force = force.data();
    fr.coord0 = coord0.data();
    fr.bcflag = bc.data();
    rc = des_write_save_host(filename, &fr);
    if (rc) return ctx_fail(c, rc, "des_write_save: cannot write %s", filename);
    return DES_OK;
}
