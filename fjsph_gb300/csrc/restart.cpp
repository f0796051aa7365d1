/*
 * restart.cpp -- restart files with the reference's content and names (src/H5IO.cpp:395-523
 * Write_Zone_Data, :1027-1060 Write_Zone_Attributes, :1092-1318 Write/Read_HDF5).
 *
 * There is no HDF5 library on this system, so the same groups, datasets and attributes go into a
 * self-describing binary container:
 *
 *   "FJSPHRST" (8 bytes), uint32 version = 1, uint32 record count, then per record
 *   uint16 name length, name bytes, uint8 kind (0 attribute, 1 dataset), uint8 type
 *   (0 f64, 1 i64, 2 i32, 3 text), uint64 element count, the elements (little endian).
 *
 * Names are the reference's: file attributes ("Simulation current time", "Current frame", ...),
 * groups "Boundary i" / "Fluid i" per block holding "Position coordinate x", "Velocity y",
 * "Acceleration z", "Pressure", "Density", "Density gradient" (the density rate), "Mass",
 * "Boundary condition", "Particle ID", "Cell ID", "Cell velocity x", "Cell density",
 * "Cell pressure", with the group's attributes as "Boundary i/Insertion normal x", ...
 * Positions are stored divided by the grid scale and read back multiplied by it, as upstream.
 * Only the public C ABI is used (download / upload of the state, settings, limits).
 */
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/fjsph_gb300.h"

namespace {

const char kMagic[8] = {'F', 'J', 'S', 'P', 'H', 'R', 'S', 'T'};
enum { kF64 = 0, kI64 = 1, kI32 = 2, kText = 3 };

struct Record {
    uint8_t kind = 0, type = 0;
    std::vector<unsigned char> bytes;
    uint64_t count = 0;
};

struct Writer {
    std::vector<std::pair<std::string, Record>> recs;
    template <typename T>
    void put(const std::string &name, uint8_t kind, uint8_t type, const T *p, uint64_t n) {
        Record r;
        r.kind = kind;
        r.type = type;
        r.count = n;
        r.bytes.resize(sizeof(T) * n);
        if (n) std::memcpy(r.bytes.data(), p, sizeof(T) * n);
        recs.emplace_back(name, std::move(r));
    }
    void attr(const std::string &name, double v) { put(name, 0, kF64, &v, 1); }
    void attr_i(const std::string &name, int64_t v) { put(name, 0, kI64, &v, 1); }
    void text(const std::string &name, const std::string &v) { put(name, 0, kText, v.data(), v.size()); }
    int save(const char *path) const {
        FILE *f = std::fopen(path, "wb");
        if (!f) return FJSPH_E_ARG;
        bool ok = std::fwrite(kMagic, 1, 8, f) == 8;
        const uint32_t version = 1, nrec = (uint32_t)recs.size();
        ok = ok && std::fwrite(&version, 4, 1, f) == 1 && std::fwrite(&nrec, 4, 1, f) == 1;
        for (const auto &kv : recs) {
            const uint16_t ln = (uint16_t)kv.first.size();
            ok = ok && std::fwrite(&ln, 2, 1, f) == 1 && std::fwrite(kv.first.data(), 1, ln, f) == ln;
            ok = ok && std::fwrite(&kv.second.kind, 1, 1, f) == 1 && std::fwrite(&kv.second.type, 1, 1, f) == 1;
            ok = ok && std::fwrite(&kv.second.count, 8, 1, f) == 1;
            ok = ok && std::fwrite(kv.second.bytes.data(), 1, kv.second.bytes.size(), f) == kv.second.bytes.size();
        }
        ok = (std::fclose(f) == 0) && ok;
        return ok ? FJSPH_OK : FJSPH_E_ARG;
    }
};

int load(const char *path, std::map<std::string, Record> &out) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return FJSPH_E_ARG;
    char magic[8];
    uint32_t version = 0, nrec = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0;
    ok = ok && std::fread(&version, 4, 1, f) == 1 && version == 1 && std::fread(&nrec, 4, 1, f) == 1;
    static const size_t esize[4] = {8, 8, 4, 1};
    for (uint32_t r = 0; ok && r < nrec; ++r) {
        uint16_t ln = 0;
        ok = std::fread(&ln, 2, 1, f) == 1;
        std::string name(ln, '\0');
        ok = ok && std::fread(&name[0], 1, ln, f) == ln;
        Record rec;
        ok = ok && std::fread(&rec.kind, 1, 1, f) == 1 && std::fread(&rec.type, 1, 1, f) == 1 && rec.type < 4;
        ok = ok && std::fread(&rec.count, 8, 1, f) == 1 && rec.count < ((uint64_t)1 << 40);
        if (!ok) break;
        rec.bytes.resize(esize[rec.type] * rec.count);
        ok = std::fread(rec.bytes.data(), 1, rec.bytes.size(), f) == rec.bytes.size();
        out[name] = std::move(rec);
    }
    std::fclose(f);
    return ok ? FJSPH_OK : FJSPH_E_ARG;
}

template <typename T>
bool get(const std::map<std::string, Record> &m, const std::string &name, uint8_t type, std::vector<T> &v) {
    auto it = m.find(name);
    if (it == m.end() || it->second.type != type) return false;
    v.resize(it->second.count);
    if (!v.empty()) std::memcpy(v.data(), it->second.bytes.data(), sizeof(T) * v.size());
    return true;
}

const char *axis(int k) { return k == 0 ? "x" : (k == 1 ? "y" : "z"); }

/* host copy of a state: every view field */
struct HostState {
    int64_t n = 0;
    int D = 3;
    std::vector<double> xi, v, acc, Af, aVisc, cellV, gradRho, norm, vPert, L;
    std::vector<double> Rrho, rho, p, m, curve, norm_curve, woccl, pDist, deltaD, cellP, cellRho, colourG, colour,
        lam, lam_nb, kernsum;
    std::vector<int64_t> part_id, cellID;
    std::vector<int32_t> b, surf, surfzone;
    void resize(int64_t n_, int D_) {
        n = n_;
        D = D_;
        for (auto *a : {&xi, &v, &acc, &Af, &aVisc, &cellV, &gradRho, &norm, &vPert}) a->assign(n * D, 0.0);
        L.assign(n * D * D, 0.0);
        for (auto *a : {&Rrho, &rho, &p, &m, &curve, &norm_curve, &woccl, &pDist, &deltaD, &cellP, &cellRho, &colourG,
                        &colour, &lam, &lam_nb, &kernsum})
            a->assign(n, 0.0);
        part_id.assign(n, 0);
        cellID.assign(n, 0);
        for (auto *a : {&b, &surf, &surfzone}) a->assign(n, 0);
    }
    fjsph_state_view view() {
        fjsph_state_view w;
        w.n = n;
        w.xi = xi.data();
        w.v = v.data();
        w.acc = acc.data();
        w.Af = Af.data();
        w.aVisc = aVisc.data();
        w.cellV = cellV.data();
        w.gradRho = gradRho.data();
        w.norm = norm.data();
        w.vPert = vPert.data();
        w.L = L.data();
        w.Rrho = Rrho.data();
        w.rho = rho.data();
        w.p = p.data();
        w.m = m.data();
        w.curve = curve.data();
        w.norm_curve = norm_curve.data();
        w.woccl = woccl.data();
        w.pDist = pDist.data();
        w.deltaD = deltaD.data();
        w.cellP = cellP.data();
        w.cellRho = cellRho.data();
        w.colourG = colourG.data();
        w.colour = colour.data();
        w.lam = lam.data();
        w.lam_nb = lam_nb.data();
        w.kernsum = kernsum.data();
        w.part_id = part_id.data();
        w.cellID = cellID.data();
        w.b = b.data();
        w.surf = surf.data();
        w.surfzone = surfzone.data();
        return w;
    }
};

std::string zone_name(const fjsph_block &B, int64_t bi, int64_t nbb) {
    return B.is_fluid ? "Fluid " + std::to_string(bi - nbb) : "Boundary " + std::to_string(bi);
}

} // namespace

extern "C" {

int fjsph_restart_write(fjsph_ctx *ctx, const char *path, int64_t current_frame) {
    if (!ctx || !path) return FJSPH_E_ARG;
    fjsph_settings s;
    int rc = fjsph_get_settings(ctx, &s);
    if (rc) return rc;
    int32_t nblk = 0;
    if ((rc = fjsph_get_limits(ctx, nullptr, 0, &nblk))) return rc;
    std::vector<fjsph_block> blocks(nblk);
    if ((rc = fjsph_get_limits(ctx, blocks.data(), nblk, &nblk))) return rc;
    int64_t n = 0, nb = 0;
    if ((rc = fjsph_particle_count(ctx, &n, &nb))) return rc;
    HostState h;
    h.resize(n, s.dim);
    fjsph_state_view view = h.view();
    if ((rc = fjsph_state_download(ctx, FJSPH_PNP1, &view))) return rc;
    int64_t nbb = 0, nfb = 0;
    for (const fjsph_block &B : blocks) (B.is_fluid ? nfb : nbb)++;
    int64_t part_next = 0;
    for (int64_t i = 0; i < n; ++i) part_next = std::max<int64_t>(part_next, h.part_id[i] + 1);
    Writer w;
    /* file attributes the restart reader uses (src/H5IO.cpp:1229-1245) */
    w.attr("Simulation current time", s.current_time);
    w.attr_i("Current frame", current_frame);
    w.attr("SPH initial spacing", s.particle_step);
    w.attr_i("Single file for output", 1);
    w.attr("SPH frame time interval", s.frame_time_interval);
    w.text("Variable list", "");
    w.attr("Grid scale", s.scale);
    w.attr("SPH CFL condition", s.cfl);
    w.attr_i("Number of boundary blocks", nbb);
    w.attr_i("Number of fluid blocks", nfb);
    w.attr_i("Number of boundary points", nb);
    w.attr_i("Number of fluid points", n - nb);
    w.attr_i("Particle index to add", part_next);
    w.attr_i("SPH stable CFL count", s.n_stable);
    w.attr_i("SPH unstable CFL count", s.n_unstable);
    const int D = s.dim;
    const double scale = s.scale != 0.0 ? s.scale : 1.0;
    for (int64_t bi = 0; bi < nblk; ++bi) {
        const fjsph_block &B = blocks[bi];
        const std::string z = zone_name(B, bi, nbb) + "/";
        const int64_t a = B.first, len = B.second - B.first;
        std::vector<double> col(len);
        auto vec = [&](const std::vector<double> &src, const char *what, double div) {
            for (int k = 0; k < D; ++k) {
                for (int64_t i = 0; i < len; ++i) col[i] = src[(a + i) * D + k] / div;
                w.put(z + what + " " + axis(k), 1, kF64, col.data(), len);
            }
        };
        auto sca = [&](const std::vector<double> &src, const char *what) {
            w.put(z + what, 1, kF64, src.data() + a, len);
        };
        vec(h.xi, "Position coordinate", scale);
        vec(h.v, "Velocity", 1.0);
        vec(h.acc, "Acceleration", 1.0);
        sca(h.p, "Pressure");
        sca(h.rho, "Density");
        sca(h.Rrho, "Density gradient");
        sca(h.m, "Mass");
        w.put(z + "Boundary condition", 1, kI32, h.b.data() + a, len);
        w.put(z + "Particle ID", 1, kI64, h.part_id.data() + a, len);
        w.put(z + "Cell ID", 1, kI64, h.cellID.data() + a, len);
        vec(h.cellV, "Cell velocity", 1.0);
        sca(h.cellRho, "Cell density");
        sca(h.cellP, "Cell pressure");
        /* zone attributes (src/H5IO.cpp:1027-1060) */
        for (int k = 0; k < 3; ++k) {
            w.attr(z + "Insertion normal " + axis(k), B.insert_norm[k]);
            w.attr(z + "Deletion normal " + axis(k), B.delete_norm[k]);
            w.attr(z + "Aerodynamic normal " + axis(k), B.aero_norm[k]);
        }
        w.attr(z + "Insertion plane constant", B.insconst);
        w.attr(z + "Deletion plane constant", B.delconst);
        w.attr(z + "Aerodynamic plane constant", B.aeroconst);
        w.attr_i(z + "Particle starting index", B.first);
        w.attr_i(z + "Particle ending index", B.second);
    }
    return w.save(path);
}

int fjsph_restart_read(fjsph_ctx *ctx, const char *path, int64_t *current_frame) {
    if (!ctx || !path) return FJSPH_E_ARG;
    std::map<std::string, Record> m;
    int rc = load(path, m);
    if (rc) return rc;
    fjsph_settings s;
    if ((rc = fjsph_get_settings(ctx, &s))) return rc;
    int32_t nblk = 0;
    if ((rc = fjsph_get_limits(ctx, nullptr, 0, &nblk))) return rc;
    std::vector<fjsph_block> blocks(nblk);
    if ((rc = fjsph_get_limits(ctx, blocks.data(), nblk, &nblk))) return rc;
    int64_t nbb = 0;
    for (const fjsph_block &B : blocks) nbb += B.is_fluid ? 0 : 1;
    std::vector<double> d1;
    std::vector<int64_t> i1;
    std::vector<int32_t> k1;
    auto num = [&](const char *name, double &out) {
        if (get(m, name, kF64, d1) && d1.size() == 1) out = d1[0];
    };
    auto inum = [&](const char *name, int64_t &out) {
        if (get(m, name, kI64, i1) && i1.size() == 1) out = i1[0];
    };
    double scale = s.scale;
    num("Grid scale", scale);
    if (scale == 0.0) scale = 1.0;
    const int64_t n = blocks.empty() ? 0 : blocks.back().second;
    const int D = s.dim;
    HostState h;
    h.resize(n, D);
    for (int64_t bi = 0; bi < nblk; ++bi) {
        const fjsph_block &B = blocks[bi];
        const std::string z = zone_name(B, bi, nbb) + "/";
        const int64_t a = B.first, len = B.second - B.first;
        auto vec = [&](std::vector<double> &dst, const char *what, double mul) -> bool {
            for (int k = 0; k < D; ++k) {
                if (!get(m, z + what + " " + axis(k), kF64, d1) || (int64_t)d1.size() != len) return false;
                for (int64_t i = 0; i < len; ++i) dst[(a + i) * D + k] = d1[i] * mul;
            }
            return true;
        };
        auto sca = [&](std::vector<double> &dst, const char *what) -> bool {
            if (!get(m, z + what, kF64, d1) || (int64_t)d1.size() != len) return false;
            std::copy(d1.begin(), d1.end(), dst.begin() + a);
            return true;
        };
        /* the block layout of the file must be the context's */
        if (!vec(h.xi, "Position coordinate", scale) || !vec(h.v, "Velocity", 1.0) || !sca(h.p, "Pressure") ||
            !sca(h.rho, "Density") || !sca(h.m, "Mass"))
            return FJSPH_E_ARG;
        vec(h.acc, "Acceleration", 1.0);
        sca(h.Rrho, "Density gradient");
        vec(h.cellV, "Cell velocity", 1.0);
        sca(h.cellRho, "Cell density");
        sca(h.cellP, "Cell pressure");
        if (!get(m, z + "Boundary condition", kI32, k1) || (int64_t)k1.size() != len) return FJSPH_E_ARG;
        std::copy(k1.begin(), k1.end(), h.b.begin() + a);
        if (get(m, z + "Particle ID", kI64, i1) && (int64_t)i1.size() == len)
            std::copy(i1.begin(), i1.end(), h.part_id.begin() + a);
        if (get(m, z + "Cell ID", kI64, i1) && (int64_t)i1.size() == len)
            std::copy(i1.begin(), i1.end(), h.cellID.begin() + a);
    }
    fjsph_state_view view = h.view();
    if ((rc = fjsph_state_upload(ctx, FJSPH_BOTH, &view))) return rc;
    /* integrator scalars (src/H5IO.cpp:1229-1245) */
    num("Simulation current time", s.current_time);
    num("SPH frame time interval", s.frame_time_interval);
    num("SPH CFL condition", s.cfl);
    int64_t ns = s.n_stable, nu = s.n_unstable, frame = 0;
    inum("SPH stable CFL count", ns);
    inum("SPH unstable CFL count", nu);
    inum("Current frame", frame);
    s.n_stable = (int32_t)ns;
    s.n_unstable = (int32_t)nu;
    if ((rc = fjsph_set_settings(ctx, &s))) return rc;
    if (current_frame) *current_frame = frame;
    return FJSPH_OK;
}

} /* extern "C" */
