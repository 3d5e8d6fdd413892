// openPMD checkpoints: the reference's Checkpoint and openPMD plugins
// (plugins/Checkpoint.x.cpp, plugins/openPMD/openPMDWriter.hpp) for the state of the
// PIC cycle (E, B, species).  Host code only: the writer and readers work on host
// arrays, and picgb_checkpoint_{write,read} move the state through the ordinary
// field and species copies of the C-ABI.
//
// One iteration is the directory <dir>/simData_<step>/: the series index
// simData_<step>.json holds the openPMD 1.1.0 tree (ED-PIC extension) in the
// attribute/dataset form of openPMD-api's JSON backend; datasets larger than a few
// values live beside it as raw little-endian C-order files named by "external".
// The index is written last, so a directory without one is an unfinished write.
#include "picgb_json.hpp"
#include "picgb_sim.hpp"

#include <cerrno>
#include <cstring>
#include <ctime>
#include <sys/stat.h>

using namespace picgb;
using namespace picgb::host;

namespace
{
    using json::Value;

    struct IoError : std::runtime_error
    {
        using std::runtime_error::runtime_error;
    };

    bool validName(char const* n)
    {
        if(!n || !n[0])
            return false;
        for(char const* p = n; *p; ++p)
        {
            char const c = *p;
            bool const ok = (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_'
                || c == '-';
            if(!ok)
                return false;
        }
        return true;
    }

    std::string iterationDir(char const* dir, uint32_t step)
    {
        return std::string(dir) + "/simData_" + std::to_string(step);
    }

    std::string indexPath(char const* dir, uint32_t step)
    {
        return iterationDir(dir, step) + "/simData_" + std::to_string(step) + ".json";
    }

    void makeDir(std::string const& p)
    {
        if(mkdir(p.c_str(), 0755) != 0 && errno != EEXIST)
            throw IoError("cannot create directory " + p + ": " + std::strerror(errno));
    }

    void writeRaw(std::string const& path, void const* data, size_t bytes)
    {
        FILE* f = std::fopen(path.c_str(), "wb");
        if(!f)
            throw IoError("cannot open " + path + " for writing: " + std::strerror(errno));
        size_t const w = bytes ? std::fwrite(data, 1, bytes, f) : 0;
        int const c = std::fclose(f);
        if(w != bytes || c != 0)
            throw IoError("short write to " + path);
    }

    void readRaw(std::string const& path, void* data, size_t bytes)
    {
        struct stat st
        {
        };
        if(stat(path.c_str(), &st) != 0)
            throw IoError("cannot stat " + path + ": " + std::strerror(errno));
        if(uint64_t(st.st_size) != uint64_t(bytes))
            throw IoError(path + " holds " + std::to_string(uint64_t(st.st_size)) + " bytes, " + std::to_string(bytes)
                          + " expected");
        FILE* f = std::fopen(path.c_str(), "rb");
        if(!f)
            throw IoError("cannot open " + path + ": " + std::strerror(errno));
        size_t const r = bytes ? std::fread(data, 1, bytes, f) : 0;
        std::fclose(f);
        if(r != bytes)
            throw IoError("short read from " + path);
    }

    std::string readText(std::string const& path)
    {
        FILE* f = std::fopen(path.c_str(), "rb");
        if(!f)
            throw IoError("cannot open " + path + ": " + std::strerror(errno));
        std::string s;
        char buf[65536];
        size_t r;
        while((r = std::fread(buf, 1, sizeof(buf), f)) > 0)
            s.append(buf, r);
        std::fclose(f);
        return s;
    }

    // ---- openPMD-api JSON-backend forms
    Value& child(Value& parent, std::string const& key)
    {
        Value& v = parent[key];
        if(!v.isObject())
            v = Value::object();
        return v;
    }

    void attr(Value& node, char const* name, Value v, char const* datatype)
    {
        Value& a = child(child(node, "attributes"), name);
        a["datatype"] = datatype;
        a["value"] = std::move(v);
    }

    Value vec(std::initializer_list<double> xs)
    {
        Value a = Value::array();
        for(double x : xs)
            a.push(x);
        return a;
    }

    Value strings(std::initializer_list<char const*> xs)
    {
        Value a = Value::array();
        for(char const* x : xs)
            a.push(x);
        return a;
    }

    // unitDimension (L, M, T, I, theta, N, J)
    Value dims(double L, double M, double T, double I) { return vec({L, M, T, I, 0.0, 0.0, 0.0}); }

    // a dataset whose data lives in `file` (relative to the iteration directory)
    void externalDataset(Value& node, char const* datatype, uint64_t extent[], int rank, std::string const& file)
    {
        node["datatype"] = datatype;
        Value e = Value::array();
        for(int i = 0; i < rank; ++i)
            e.push(extent[i]);
        node["extent"] = std::move(e);
        node["external"] = file;
    }

    // a one-element dataset held inline
    void inlineDataset(Value& node, char const* datatype, double value)
    {
        node["datatype"] = datatype;
        Value d = Value::array();
        d.push(value);
        node["data"] = std::move(d);
    }

    void recordAttrs(Value& rec, Value unitDimension, int macroWeighted, double weightingPower)
    {
        attr(rec, "unitDimension", std::move(unitDimension), "ARR_DBL_7");
        attr(rec, "timeOffset", 0.0, "FLOAT");
        attr(rec, "macroWeighted", unsigned(macroWeighted), "UINT");
        attr(rec, "weightingPower", weightingPower, "DOUBLE");
    }

    char const* pusherName(int p)
    {
        switch(p)
        {
        case PICGB_PUSHER_BORIS:
            return "Boris";
        case PICGB_PUSHER_HIGUERA_CARY:
            return "HigueraCary";
        case PICGB_PUSHER_VAY:
            return "Vay";
        case PICGB_PUSHER_FREE:
            return "Free";
        default:
            return "none";
        }
    }

    std::string utcDate()
    {
        std::time_t const t = std::time(nullptr);
        std::tm tm{};
        gmtime_r(&t, &tm);
        char buf[64];
        std::strftime(buf, sizeof(buf), "%Y-%m-%d %H:%M:%S +0000", &tm);
        return buf;
    }

    // Yee staggering of the components in (z, y, x) order (fields/YeeCell.hpp:70-131)
    constexpr float kStagE[3][3] = {{0.f, 0.f, 0.5f}, {0.f, 0.5f, 0.f}, {0.5f, 0.f, 0.f}};
    constexpr float kStagB[3][3] = {{0.5f, 0.5f, 0.f}, {0.5f, 0.f, 0.5f}, {0.f, 0.5f, 0.5f}};
    char const* const kComp[3] = {"x", "y", "z"};

    void checkGrid(picgb_grid_config const* g, int sc[3])
    {
        if(!g)
            throw std::invalid_argument("null grid");
        if(!scSize(g->supercell, sc))
            throw std::invalid_argument("unknown supercell id " + std::to_string(g->supercell));
        if(g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || g->nx % sc[0] || g->ny % sc[1] || g->nz % sc[2])
            throw std::invalid_argument("grid is not a positive multiple of the supercell");
    }

    // ---- the writer
    // names of the six components of a PML convolution field (psi.ab: field component a,
    // derivative along b), in the order of the device arrays
    char const* const kPsiNames[6] = {"xy", "xz", "yx", "yz", "zx", "zy"};

    // psiE, psiB: the PML convolution fields (6 host arrays of nx*ny*nz floats each) written as
    // the extra meshes "PmlPsiE" and "PmlPsiB", or null
    void writeSeries(
        char const* dir,
        uint32_t step,
        picgb_grid_config const& g,
        float const* const* E,
        float const* const* B,
        int nspecies,
        picgb_openpmd_species const* species,
        float const* const* psiE = nullptr,
        float const* const* psiB = nullptr)
    {
        int sc[3];
        checkGrid(&g, sc);
        if(!dir || !dir[0])
            throw std::invalid_argument("null directory");
        if(!E || !B || (nspecies > 0 && !species) || nspecies < 0)
            throw std::invalid_argument("null field or species arrays");
        for(int c = 0; c < 3; ++c)
            if(!E[c] || !B[c])
                throw std::invalid_argument("null field component");
        for(int s = 0; s < nspecies; ++s)
        {
            if(!validName(species[s].name))
                throw std::invalid_argument("species name must be letters, digits, '_' or '-'");
            for(int t = 0; t < s; ++t)
                if(std::strcmp(species[s].name, species[t].name) == 0)
                    throw std::invalid_argument(std::string("species '") + species[s].name + "' given twice");
            picgb_particles const& p = species[s].particles;
            if(p.n > 0 && (!p.pos[0] || !p.pos[1] || !p.pos[2] || !p.mom[0] || !p.mom[1] || !p.mom[2] || !p.w || !p.sc
                           || !p.lcell))
                throw std::invalid_argument(std::string("species '") + species[s].name + "': null particle array");
        }
        makeDir(dir);
        std::string const base = iterationDir(dir, step);
        makeDir(base);
        uint64_t const ncell = uint64_t(g.nx) * g.ny * g.nz;
        uint64_t meshExtent[3] = {uint64_t(g.nz), uint64_t(g.ny), uint64_t(g.nx)};

        Value root = Value::object();
        attr(root, "openPMD", "1.1.0", "STRING");
        attr(root, "openPMDextension", 1u, "UINT"); // ED-PIC
        attr(root, "basePath", "/data/%T/", "STRING");
        attr(root, "meshesPath", "meshes/", "STRING");
        attr(root, "particlesPath", "particles/", "STRING");
        attr(root, "iterationEncoding", "fileBased", "STRING");
        attr(root, "iterationFormat", "simData_%T", "STRING");
        attr(root, "software", "picongpu_gb300", "STRING");
        attr(root, "softwareVersion", std::to_string(PICGB_ABI_VERSION), "STRING");
        attr(root, "date", utcDate(), "STRING");
        Value& it = child(child(root, "data"), std::to_string(step));
        attr(it, "dt", double(g.dt), "DOUBLE");
        attr(it, "time", double(step) * double(g.dt), "DOUBLE");
        attr(it, "timeUnitSI", 1.0, "DOUBLE");

        Value& meshes = child(it, "meshes");
        attr(meshes, "fieldSolver", "Yee", "STRING");
        attr(meshes, "fieldBoundary", strings({"periodic", "periodic", "periodic", "periodic", "periodic", "periodic"}),
             "VEC_STRING");
        attr(meshes, "particleBoundary",
             strings({"periodic", "periodic", "periodic", "periodic", "periodic", "periodic"}), "VEC_STRING");
        attr(meshes, "currentSmoothing", "none", "STRING");
        attr(meshes, "chargeCorrection", "none", "STRING");
        for(int f = 0; f < 2; ++f)
        {
            char const* name = f == 0 ? "E" : "B";
            float const* const* data = f == 0 ? E : B;
            Value& m = child(meshes, name);
            attr(m, "geometry", "cartesian", "STRING");
            attr(m, "dataOrder", "C", "STRING");
            attr(m, "axisLabels", strings({"z", "y", "x"}), "VEC_STRING");
            attr(m, "gridSpacing", vec({g.dz, g.dy, g.dx}), "VEC_DOUBLE");
            attr(m, "gridGlobalOffset", vec({0.0, 0.0, 0.0}), "VEC_DOUBLE");
            attr(m, "gridUnitSI", 1.0, "DOUBLE");
            attr(m, "unitDimension", f == 0 ? dims(1, 1, -3, -1) : dims(0, 1, -2, -1), "ARR_DBL_7");
            attr(m, "timeOffset", 0.0, "FLOAT");
            attr(m, "fieldSmoothing", "none", "STRING");
            for(int c = 0; c < 3; ++c)
            {
                Value& comp = child(m, kComp[c]);
                float const* st = f == 0 ? kStagE[c] : kStagB[c];
                attr(comp, "position", vec({st[0], st[1], st[2]}), "VEC_FLOAT");
                attr(comp, "unitSI", 1.0, "DOUBLE");
                std::string const file = std::string("meshes_") + name + "_" + kComp[c] + ".bin";
                externalDataset(comp, "FLOAT", meshExtent, 3, file);
                writeRaw(base + "/" + file, data[c], sizeof(float) * ncell);
            }
        }

        for(int f = 0; f < 2 && psiE && psiB; ++f)
        {
            // not an openPMD record of the reference: the state of the open boundaries' PML
            char const* name = f == 0 ? "PmlPsiE" : "PmlPsiB";
            float const* const* data = f == 0 ? psiE : psiB;
            Value& m = child(meshes, name);
            attr(m, "geometry", "cartesian", "STRING");
            attr(m, "dataOrder", "C", "STRING");
            attr(m, "axisLabels", strings({"z", "y", "x"}), "VEC_STRING");
            attr(m, "gridSpacing", vec({g.dz, g.dy, g.dx}), "VEC_DOUBLE");
            attr(m, "gridGlobalOffset", vec({0.0, 0.0, 0.0}), "VEC_DOUBLE");
            attr(m, "gridUnitSI", 1.0, "DOUBLE");
            attr(m, "unitDimension", f == 0 ? dims(1, 1, -3, -1) : dims(0, 1, -2, -1), "ARR_DBL_7");
            attr(m, "timeOffset", 0.0, "FLOAT");
            for(int c = 0; c < 6; ++c)
            {
                Value& comp = child(m, kPsiNames[c]);
                float const* st = f == 0 ? kStagE[c / 2] : kStagB[c / 2];
                attr(comp, "position", vec({st[0], st[1], st[2]}), "VEC_FLOAT");
                attr(comp, "unitSI", 1.0, "DOUBLE");
                std::string const file = std::string("meshes_") + name + "_" + kPsiNames[c] + ".bin";
                externalDataset(comp, "FLOAT", meshExtent, 3, file);
                writeRaw(base + "/" + file, data[c], sizeof(float) * ncell);
            }
        }

        Value& particles = child(it, "particles");
        double const cellEdge[3] = {g.dx, g.dy, g.dz};
        for(int s = 0; s < nspecies; ++s)
        {
            picgb_openpmd_species const& sp = species[s];
            picgb_particles const& p = sp.particles;
            uint64_t n[1] = {p.n};
            std::string const pre = std::string("particles_") + sp.name + "_";
            Value& ps = child(particles, sp.name);
            attr(ps, "particleShape", double(sp.shape), "FLOAT");
            attr(ps, "currentDeposition",
                 sp.current == PICGB_CURRENT_ESIRKEPOV ? "Esirkepov" : (sp.current == PICGB_CURRENT_EMZ ? "EmZ" : "none"),
                 "STRING");
            attr(ps, "particlePush", pusherName(sp.pusher), "STRING");
            attr(ps, "particleInterpolation", "uniform", "STRING");
            attr(ps, "particleSmoothing", "none", "STRING");

            // global cell index of every particle from (supercell, cell in supercell)
            std::vector<int32_t> off[3];
            for(auto& o : off)
                o.resize(p.n);
            int const nscx = g.nx / sc[0], nscy = g.ny / sc[1];
            int const nsc = nscx * nscy * (g.nz / sc[2]);
            int const vol = sc[0] * sc[1] * sc[2];
            for(uint64_t k = 0; k < p.n; ++k)
            {
                int32_t const q = p.sc[k];
                int const lc = p.lcell[k];
                if(q < 0 || q >= nsc || lc >= vol)
                    throw std::invalid_argument(std::string("species '") + sp.name + "': supercell or cell index out of range");
                off[0][k] = (q % nscx) * sc[0] + lc % sc[0];
                off[1][k] = ((q / nscx) % nscy) * sc[1] + (lc / sc[0]) % sc[1];
                off[2][k] = (q / (nscx * nscy)) * sc[2] + lc / (sc[0] * sc[1]);
            }

            // position (in-cell, in cell edges), positionOffset (cell index), momentum
            for(int r = 0; r < 3; ++r)
            {
                char const* const rname[3] = {"position", "positionOffset", "momentum"};
                Value& rec = child(ps, rname[r]);
                recordAttrs(rec, r < 2 ? dims(1, 0, 0, 0) : dims(1, 1, -1, 0), r < 2 ? 0 : 1, r < 2 ? 0.0 : 1.0);
                for(int c = 0; c < 3; ++c)
                {
                    Value& comp = child(rec, kComp[c]);
                    attr(comp, "unitSI", r < 2 ? cellEdge[c] : 1.0, "DOUBLE");
                    std::string const file = pre + rname[r] + "_" + kComp[c] + ".bin";
                    externalDataset(comp, r == 1 ? "INT" : "FLOAT", n, 1, file);
                    void const* data = r == 0 ? static_cast<void const*>(p.pos[c])
                                              : (r == 1 ? static_cast<void const*>(off[c].data()) : p.mom[c]);
                    writeRaw(base + "/" + file, data, 4 * p.n);
                }
            }
            Value& w = child(ps, "weighting");
            recordAttrs(w, dims(0, 0, 0, 0), 1, 1.0);
            attr(w, "unitSI", 1.0, "DOUBLE");
            externalDataset(w, "FLOAT", n, 1, pre + "weighting.bin");
            writeRaw(base + "/" + pre + "weighting.bin", p.w, sizeof(float) * p.n);
            for(int k = 0; k < 2; ++k)
            {
                // constant records (openPMD 1.1.0 "constant record components")
                Value& r = child(ps, k == 0 ? "charge" : "mass");
                recordAttrs(r, k == 0 ? dims(0, 0, 1, 1) : dims(0, 1, 0, 0), 0, 1.0);
                attr(r, "value", double(k == 0 ? sp.charge : sp.mass), "FLOAT");
                Value shape = Value::array();
                shape.push(p.n);
                attr(r, "shape", std::move(shape), "VEC_ULONG");
                attr(r, "unitSI", 1.0, "DOUBLE");
            }
            if(p.id && p.n > 0)
            {
                Value& id = child(ps, "id");
                recordAttrs(id, dims(0, 0, 0, 0), 0, 0.0);
                attr(id, "unitSI", 1.0, "DOUBLE");
                externalDataset(id, "UINT", n, 1, pre + "id.bin");
                writeRaw(base + "/" + pre + "id.bin", p.id, sizeof(uint32_t) * p.n);
            }
            // one particle patch covering the box (the reference writes one per GPU)
            Value& pp = child(ps, "particlePatches");
            Value& np = child(pp, "numParticles");
            attr(np, "unitSI", 1.0, "DOUBLE");
            inlineDataset(np, "ULONG", double(p.n));
            Value& npo = child(pp, "numParticlesOffset");
            attr(npo, "unitSI", 1.0, "DOUBLE");
            inlineDataset(npo, "ULONG", 0.0);
            int const cells[3] = {g.nx, g.ny, g.nz};
            for(int k = 0; k < 2; ++k)
            {
                Value& r = child(pp, k == 0 ? "offset" : "extent");
                attr(r, "unitDimension", dims(1, 0, 0, 0), "ARR_DBL_7");
                for(int c = 0; c < 3; ++c)
                {
                    Value& comp = child(r, kComp[c]);
                    attr(comp, "unitSI", cellEdge[c], "DOUBLE");
                    inlineDataset(comp, "ULONG", k == 0 ? 0.0 : double(cells[c]));
                }
            }
        }

        std::string text;
        root.write(text);
        text += '\n';
        writeRaw(indexPath(dir, step), text.data(), text.size());
    }

    // ---- the readers
    struct Index
    {
        Value root;
        Value const* it = nullptr; // data/<step>
    };

    Index openIndex(char const* dir, uint32_t step)
    {
        if(!dir || !dir[0])
            throw std::invalid_argument("null directory");
        Index x;
        x.root = Value::parse(readText(indexPath(dir, step)));
        Value const* ver = x.root.at("attributes").find("openPMD");
        if(!ver || ver->at("value").string().rfind("1.", 0) != 0)
            throw IoError("not an openPMD 1.x series index");
        x.it = x.root.at("data").find(std::to_string(step));
        if(!x.it)
            throw IoError("iteration " + std::to_string(step) + " is not in the series index");
        return x;
    }

    uint64_t extent1(Value const& ds)
    {
        auto const& e = ds.at("extent").items();
        if(e.size() != 1)
            throw IoError("expected a one-dimensional particle dataset");
        return uint64_t(e[0].number());
    }

    void readExternal(
        char const* dir,
        uint32_t step,
        Value const& ds,
        char const* datatype,
        void* dst,
        size_t elemBytes,
        uint64_t count)
    {
        if(ds.at("datatype").string() != datatype)
            throw IoError(std::string("dataset datatype ") + ds.at("datatype").string() + ", " + datatype + " expected");
        std::string const& file = ds.at("external").string();
        if(file.find('/') != std::string::npos || file.find("..") != std::string::npos)
            throw IoError("dataset file name " + file + " leaves the iteration directory");
        readRaw(iterationDir(dir, step) + "/" + file, dst, elemBytes * count);
    }

    Value const& speciesNode(Index const& x, char const* name)
    {
        Value const* ps = x.it->find("particles");
        Value const* s = ps ? ps->find(name) : nullptr;
        if(!s)
            throw std::out_of_range(std::string("species '") + name + "' is not in the checkpoint");
        return *s;
    }

    uint64_t speciesCount(Index const& x, char const* name)
    {
        return extent1(speciesNode(x, name).at("position").at("x"));
    }

    void readSpecies(
        char const* dir,
        uint32_t step,
        char const* name,
        picgb_grid_config const* g,
        picgb_particles* h)
    {
        int sc[3];
        checkGrid(g, sc);
        if(!h || !validName(name))
            throw std::invalid_argument("null host arrays or invalid species name");
        Index const x = openIndex(dir, step);
        Value const& s = speciesNode(x, name);
        uint64_t const n = speciesCount(x, name);
        if(h->n < n)
            throw std::invalid_argument("host arrays hold " + std::to_string(h->n) + " particles, " + std::to_string(n)
                                        + " needed");
        if(n > 0
           && (!h->pos[0] || !h->pos[1] || !h->pos[2] || !h->mom[0] || !h->mom[1] || !h->mom[2] || !h->w || !h->sc
               || !h->lcell))
            throw std::invalid_argument("null host particle array");
        Value const* idRec = s.find("id");
        if(h->id && n > 0 && !idRec)
            throw std::out_of_range(std::string("species '") + name + "' has no id record");
        std::vector<int32_t> off[3];
        int const cells[3] = {g->nx, g->ny, g->nz};
        for(int c = 0; c < 3; ++c)
        {
            if(extent1(s.at("position").at(kComp[c])) != n || extent1(s.at("momentum").at(kComp[c])) != n
               || extent1(s.at("positionOffset").at(kComp[c])) != n)
                throw IoError("particle records of unequal length");
            readExternal(dir, step, s.at("position").at(kComp[c]), "FLOAT", h->pos[c], sizeof(float), n);
            readExternal(dir, step, s.at("momentum").at(kComp[c]), "FLOAT", h->mom[c], sizeof(float), n);
            off[c].resize(n);
            readExternal(dir, step, s.at("positionOffset").at(kComp[c]), "INT", off[c].data(), sizeof(int32_t), n);
        }
        if(extent1(s.at("weighting")) != n)
            throw IoError("particle records of unequal length");
        readExternal(dir, step, s.at("weighting"), "FLOAT", h->w, sizeof(float), n);
        if(h->id && n > 0)
        {
            if(extent1(*idRec) != n)
                throw IoError("particle records of unequal length");
            readExternal(dir, step, *idRec, "UINT", h->id, sizeof(uint32_t), n);
        }
        int const nscx = g->nx / sc[0], nscy = g->ny / sc[1];
        for(uint64_t k = 0; k < n; ++k)
        {
            int q[3], l[3];
            for(int c = 0; c < 3; ++c)
            {
                int32_t const v = off[c][k];
                if(v < 0 || v >= cells[c])
                    throw IoError("positionOffset outside the grid: the checkpoint's grid differs");
                q[c] = v / sc[c];
                l[c] = v % sc[c];
            }
            h->sc[k] = q[0] + nscx * (q[1] + nscy * q[2]);
            h->lcell[k] = uint16_t(l[0] + sc[0] * (l[1] + sc[1] * l[2]));
        }
        h->n = n;
    }

    // Reads the components `comps` of mesh `name`; returns false when the mesh is absent and
    // `optional` is set.
    bool readMeshComponents(
        char const* dir,
        uint32_t step,
        char const* name,
        picgb_grid_config const* g,
        float* const* host,
        char const* const* comps,
        int ncomp,
        bool optional)
    {
        int sc[3];
        checkGrid(g, sc);
        Index const x = openIndex(dir, step);
        Value const* ms = x.it->find("meshes");
        Value const* m = ms ? ms->find(name) : nullptr;
        if(!m)
        {
            if(optional)
                return false;
            throw std::out_of_range(std::string("mesh '") + name + "' is not in the checkpoint");
        }
        uint64_t const ncell = uint64_t(g->nx) * g->ny * g->nz;
        double const want[3] = {double(g->nz), double(g->ny), double(g->nx)};
        for(int c = 0; c < ncomp; ++c)
        {
            Value const& comp = m->at(comps[c]);
            auto const& e = comp.at("extent").items();
            if(e.size() != 3 || e[0].number() != want[0] || e[1].number() != want[1] || e[2].number() != want[2])
                throw IoError(std::string("mesh ") + name + " has another extent than the grid");
            readExternal(dir, step, comp, "FLOAT", host[c], sizeof(float), ncell);
        }
        return true;
    }

    void readMesh(char const* dir, uint32_t step, char const* name, picgb_grid_config const* g, float* const* host)
    {
        int sc[3];
        checkGrid(g, sc);
        if(!host || !name || (std::strcmp(name, "E") != 0 && std::strcmp(name, "B") != 0))
            throw std::invalid_argument("mesh name must be \"E\" or \"B\"");
        for(int c = 0; c < 3; ++c)
            if(!host[c])
                throw std::invalid_argument("null host field component");
        Index const x = openIndex(dir, step);
        Value const* ms = x.it->find("meshes");
        Value const* m = ms ? ms->find(name) : nullptr;
        if(!m)
            throw std::out_of_range(std::string("mesh '") + name + "' is not in the checkpoint");
        if(m->at("attributes").at("dataOrder").at("value").string() != "C")
            throw IoError("only dataOrder C is read");
        uint64_t const ncell = uint64_t(g->nx) * g->ny * g->nz;
        double const want[3] = {double(g->nz), double(g->ny), double(g->nx)};
        for(int c = 0; c < 3; ++c)
        {
            Value const& comp = m->at(kComp[c]);
            auto const& e = comp.at("extent").items();
            if(e.size() != 3 || e[0].number() != want[0] || e[1].number() != want[1] || e[2].number() != want[2])
                throw IoError(std::string("mesh ") + name + " has another extent than the grid");
            readExternal(dir, step, comp, "FLOAT", host[c], sizeof(float), ncell);
        }
    }

    // Runs `f`, turning exceptions into status codes and the thread's error message.
    template<typename F>
    int guarded(char const* what, F&& f)
    {
        try
        {
            return f();
        }
        catch(std::invalid_argument const& e)
        {
            return fail(PICGB_ERR_INVALID, "%s: %s", what, e.what());
        }
        catch(std::out_of_range const& e)
        {
            return fail(PICGB_ERR_NOT_FOUND, "%s: %s", what, e.what());
        }
        catch(std::bad_alloc const&)
        {
            return fail(PICGB_ERR_IO, "%s: out of host memory", what);
        }
        catch(std::exception const& e)
        {
            return fail(PICGB_ERR_IO, "%s: %s", what, e.what());
        }
    }
} // namespace

extern "C"
{
    int picgb_openpmd_write(
        const char* dir,
        uint32_t step,
        const picgb_grid_config* grid,
        const float* const* E,
        const float* const* B,
        int32_t nspecies,
        const picgb_openpmd_species* species)
    {
        return guarded(
            "openPMD write",
            [&]
            {
                if(!grid)
                    throw std::invalid_argument("null grid");
                writeSeries(dir, step, *grid, E, B, nspecies, species);
                return int(PICGB_OK);
            });
    }

    int picgb_openpmd_species_count(const char* dir, uint32_t step, const char* name, uint64_t* n)
    {
        return guarded(
            "openPMD read",
            [&]
            {
                if(!n || !validName(name))
                    throw std::invalid_argument("null count or invalid species name");
                *n = speciesCount(openIndex(dir, step), name);
                return int(PICGB_OK);
            });
    }

    int picgb_openpmd_read_species(
        const char* dir,
        uint32_t step,
        const char* name,
        const picgb_grid_config* grid,
        picgb_particles* host)
    {
        return guarded(
            "openPMD read",
            [&]
            {
                readSpecies(dir, step, name, grid, host);
                return int(PICGB_OK);
            });
    }

    int picgb_openpmd_read_mesh(
        const char* dir,
        uint32_t step,
        const char* name,
        const picgb_grid_config* grid,
        float* const* host)
    {
        return guarded(
            "openPMD read",
            [&]
            {
                readMesh(dir, step, name, grid, host);
                return int(PICGB_OK);
            });
    }

    int picgb_checkpoint_write(picgb_sim* s, const char* dir, uint32_t step)
    {
        if(int r = checkSim(s))
            return r;
        return guarded(
            "checkpoint write",
            [&]
            {
                size_t const ncell = s->ncell;
                std::vector<float> fE(3 * ncell), fB(3 * ncell);
                float* pe[3] = {fE.data(), fE.data() + ncell, fE.data() + 2 * ncell};
                float* pb[3] = {fB.data(), fB.data() + ncell, fB.data() + 2 * ncell};
                if(int r = picgb_field_get(s, "E", pe))
                    return r;
                if(int r = picgb_field_get(s, "B", pb))
                    return r;
                // host arrays per species: 7 float rows, sc, lcell, id
                struct Host
                {
                    std::vector<float> a;
                    std::vector<int32_t> sc;
                    std::vector<uint16_t> lcell;
                    std::vector<uint32_t> id;
                };
                std::vector<Host> hosts(s->species.size());
                std::vector<picgb_openpmd_species> out(s->species.size());
                for(size_t i = 0; i < s->species.size(); ++i)
                {
                    Species const& sp = *s->species[i];
                    uint64_t n = 0;
                    if(int r = picgb_species_count(s, int32_t(i), &n))
                        return r;
                    Host& h = hosts[i];
                    h.a.resize(7 * n);
                    h.sc.resize(n);
                    h.lcell.resize(n);
                    if(sp.cfg.with_ids)
                        h.id.resize(n);
                    picgb_openpmd_species& o = out[i];
                    o.name = sp.name.c_str();
                    o.charge = sp.cfg.charge;
                    o.mass = sp.cfg.mass;
                    o.pusher = sp.cfg.pusher;
                    o.shape = sp.cfg.shape;
                    o.current = sp.cfg.current;
                    picgb_particles& p = o.particles;
                    p.n = n;
                    for(int c = 0; c < 3; ++c)
                    {
                        p.pos[c] = h.a.data() + c * n;
                        p.mom[c] = h.a.data() + (3 + c) * n;
                    }
                    p.w = h.a.data() + 6 * n;
                    p.sc = h.sc.data();
                    p.lcell = h.lcell.data();
                    p.id = sp.cfg.with_ids ? h.id.data() : nullptr;
                    if(n > 0)
                        if(int r = picgb_species_get(s, int32_t(i), &p))
                            return r;
                }
                // the PML convolution fields of open boundaries, so that a restart continues exactly
                std::vector<float> psi;
                float* qe[6] = {};
                float* qb[6] = {};
                if(s->g.open && s->pml.psiE)
                {
                    psi.resize(12 * ncell);
                    CUDA_TRY(cudaMemcpyAsync(psi.data(), s->pml.psiE, sizeof(float) * 6 * ncell, cudaMemcpyDeviceToHost, s->stream));
                    CUDA_TRY(cudaMemcpyAsync(psi.data() + 6 * ncell, s->pml.psiB, sizeof(float) * 6 * ncell, cudaMemcpyDeviceToHost,
                                             s->stream));
                    CUDA_TRY(cudaStreamSynchronize(s->stream));
                    for(int c = 0; c < 6; ++c)
                    {
                        qe[c] = psi.data() + c * ncell;
                        qb[c] = psi.data() + (6 + c) * ncell;
                    }
                }
                bool const withPsi = s->g.open && s->pml.psiE;
                writeSeries(dir, step, s->cfg, pe, pb, int(out.size()), out.data(), withPsi ? qe : nullptr,
                            withPsi ? qb : nullptr);
                return int(PICGB_OK);
            });
    }

    int picgb_checkpoint_read(picgb_sim* s, const char* dir, uint32_t step)
    {
        if(int r = checkSim(s))
            return r;
        return guarded(
            "checkpoint read",
            [&]
            {
                size_t const ncell = s->ncell;
                std::vector<float> f(3 * ncell);
                float* p3[3] = {f.data(), f.data() + ncell, f.data() + 2 * ncell};
                for(char const* name : {"E", "B"})
                {
                    readMesh(dir, step, name, &s->cfg, p3);
                    if(int r = picgb_field_set(s, name, p3))
                        return r;
                }
                std::fill(f.begin(), f.end(), 0.0f);
                if(int r = picgb_field_set(s, "J", p3))
                    return r;
                if(s->g.open && s->pml.psiE)
                {
                    // PML state of the checkpoint if it has one (set_boundaries zeroed it before)
                    std::vector<float> psi(6 * ncell);
                    float* q[6];
                    for(int c = 0; c < 6; ++c)
                        q[c] = psi.data() + c * ncell;
                    for(int fld = 0; fld < 2; ++fld)
                        if(readMeshComponents(dir, step, fld == 0 ? "PmlPsiE" : "PmlPsiB", &s->cfg, q, kPsiNames, 6, true))
                        {
                            CUDA_TRY(cudaMemcpyAsync(fld == 0 ? s->pml.psiE : s->pml.psiB, psi.data(), sizeof(float) * 6 * ncell,
                                                     cudaMemcpyHostToDevice, s->stream));
                            CUDA_TRY(cudaStreamSynchronize(s->stream));
                        }
                }
                Index const x = openIndex(dir, step);
                for(size_t i = 0; i < s->species.size(); ++i)
                {
                    Species const& sp = *s->species[i];
                    uint64_t const n = speciesCount(x, sp.name.c_str());
                    std::vector<float> a(7 * n);
                    std::vector<int32_t> scv(n);
                    std::vector<uint16_t> lc(n);
                    std::vector<uint32_t> id(sp.cfg.with_ids ? n : 0);
                    picgb_particles p{};
                    p.n = n;
                    for(int c = 0; c < 3; ++c)
                    {
                        p.pos[c] = a.data() + c * n;
                        p.mom[c] = a.data() + (3 + c) * n;
                    }
                    p.w = a.data() + 6 * n;
                    p.sc = scv.data();
                    p.lcell = lc.data();
                    p.id = sp.cfg.with_ids ? id.data() : nullptr;
                    readSpecies(dir, step, sp.name.c_str(), &s->cfg, &p);
                    if(int r = picgb_species_set(s, int32_t(i), &p))
                        return r;
                }
                return int(PICGB_OK);
            });
    }
}
