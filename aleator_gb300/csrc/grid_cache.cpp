// The reference's on-disk FrameworkEnergyGrid cache format, version 1
// (engines/monte_carlo/framework_energy_grid.cc:24-138, 290-409): a grid built
// on the GPU is written to, and read from, the same bytes the reference CPU
// build writes, under the same content-addressed file name, so either side
// can reuse the other's cache.
//
// Layout (little-endian, native widths):
//   u32 version (1)
//   key: u64 n + n f64 atomX | atomY | atomZ ; u64 n + n u32 atomSpecies ;
//        9 f64 lattice (row-major) ; u64 n_lj + n_lj x (f64 eps, f64 sigma) ;
//        f64 cutoff ; u8 truncation ; u64 n + n u32 sorted distinct guests ;
//        f64 spacing ; f64 energy cap (1e5)
//   i32 nx, ny, nz ; u64 n_tables ; n_tables x (u32 species, u64 n, n f64)
// File name: framework_energy_grid_v1_<FNV-1a 64 of the key bytes, %016llx>.bin
//
// Table order: the reference iterates an std::unordered_map<uint32_t, Table>
// (framework_energy_grid.cc:309). With libstdc++ and the few guest species a
// grid carries (each in its own bucket, no rehash after the first insert)
// that order is the reverse of insertion, i.e. descending species id, which
// is the order written here. That order is an accident of one standard
// library, so the reader does not rely on it: it accepts the tables in any
// order and sorts them by species id.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "grid.cuh"

namespace alea {

namespace {

constexpr uint32_t kVersion = 1;

struct Key {
    std::vector<double> x, y, z;
    std::vector<uint32_t> species;
    double lattice[9];
    std::vector<double> eps, sigma;
    double cutoff;
    uint8_t truncation;
    std::vector<uint32_t> guests;
    double spacing;
    double cap;
    bool operator==(const Key& o) const {
        return x == o.x && y == o.y && z == o.z && species == o.species &&
               std::memcmp(lattice, o.lattice, sizeof lattice) == 0 && eps == o.eps &&
               sigma == o.sigma && cutoff == o.cutoff && truncation == o.truncation &&
               guests == o.guests && spacing == o.spacing && cap == o.cap;
    }
};

// makeFrameworkEnergyGridCacheKey (framework_energy_grid.cc:169-191)
Key make_key(const alea_lennard_jones& lj, const alea_particles& fw, const alea_lattice& lat,
             const uint32_t* guest, uint32_t n_guest, double spacing) {
    Key k;
    k.x.assign(fw.x, fw.x + fw.n);
    k.y.assign(fw.y, fw.y + fw.n);
    k.z.assign(fw.z, fw.z + fw.n);
    k.species.resize(fw.n, 0);
    if (fw.species) k.species.assign(fw.species, fw.species + fw.n);
    std::memcpy(k.lattice, lat.m, sizeof k.lattice);
    k.eps.assign(lj.epsilon, lj.epsilon + lj.n_species);
    k.sigma.assign(lj.sigma, lj.sigma + lj.n_species);
    k.cutoff = lj.cutoff;
    k.truncation = (uint8_t)lj.truncation;
    k.guests.assign(guest, guest + n_guest);
    std::sort(k.guests.begin(), k.guests.end());
    k.guests.erase(std::unique(k.guests.begin(), k.guests.end()), k.guests.end());
    k.spacing = spacing;
    k.cap = kEnergyCap;
    return k;
}

template <typename T>
void put(std::string& b, const T& v) {
    b.append(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <typename T>
void put_vec(std::string& b, const std::vector<T>& v) {
    put(b, (uint64_t)v.size());
    if (!v.empty()) b.append(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

// writeKey (framework_energy_grid.cc:77-97)
std::string key_bytes(const Key& k) {
    std::string b;
    put_vec(b, k.x);
    put_vec(b, k.y);
    put_vec(b, k.z);
    put_vec(b, k.species);
    for (double v : k.lattice) put(b, v);
    put(b, (uint64_t)k.eps.size());
    for (size_t i = 0; i < k.eps.size(); ++i) {
        put(b, k.eps[i]);
        put(b, k.sigma[i]);
    }
    put(b, k.cutoff);
    put(b, k.truncation);
    put_vec(b, k.guests);
    put(b, k.spacing);
    put(b, k.cap);
    return b;
}

// framework_energy_grid.cc:128-138
uint64_t fnv1a64(const std::string& s) {
    uint64_t h = 0xcbf29ce484222325ULL;
    for (unsigned char c : s) {
        h ^= (uint64_t)c;
        h *= 0x100000001b3ULL;
    }
    return h;
}

std::string file_name(const Key& k) {
    char hex[17];
    std::snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a64(key_bytes(k)));
    return "framework_energy_grid_v" + std::to_string(kVersion) + "_" + hex + ".bin";
}

struct Reader {
    std::ifstream& in;
    template <typename T>
    T get() {
        T v{};
        in.read(reinterpret_cast<char*>(&v), sizeof(T));
        return v;
    }
    template <typename T>
    std::vector<T> get_vec(uint64_t limit) {
        const uint64_t n = get<uint64_t>();
        if (!in || n > limit) {
            in.setstate(std::ios::failbit);
            return {};
        }
        std::vector<T> v(n);
        if (n) in.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
        return v;
    }
};

// readKey (framework_energy_grid.cc:99-123); vector lengths are bounded by the
// file size so a corrupt length fails as a truncated read.
Key read_key(Reader& r, uint64_t limit) {
    Key k;
    k.x = r.get_vec<double>(limit);
    k.y = r.get_vec<double>(limit);
    k.z = r.get_vec<double>(limit);
    k.species = r.get_vec<uint32_t>(limit);
    for (double& v : k.lattice) v = r.get<double>();
    const uint64_t ns = r.get<uint64_t>();
    if (!r.in || ns > limit) {
        r.in.setstate(std::ios::failbit);
        return k;
    }
    k.eps.resize(ns);
    k.sigma.resize(ns);
    for (uint64_t i = 0; i < ns; ++i) {
        k.eps[i] = r.get<double>();
        k.sigma[i] = r.get<double>();
    }
    k.cutoff = r.get<double>();
    k.truncation = r.get<uint8_t>();
    k.guests = r.get_vec<uint32_t>(limit);
    k.spacing = r.get<double>();
    k.cap = r.get<double>();
    return k;
}

}  // namespace

std::string grid_cache_file_name(const alea_lennard_jones& lj, const alea_particles& fw,
                                 const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                                 double spacing) {
    return file_name(make_key(lj, fw, lat, guest, n_guest, spacing));
}

// serialize (framework_energy_grid.cc:290-316)
void grid_cache_write(const char* path, const alea_lennard_jones& lj, const alea_particles& fw,
                      const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                      double spacing, const int32_t counts[3], const std::vector<uint32_t>& species,
                      const std::vector<std::vector<double>>& tables) {
    const Key k = make_key(lj, fw, lat, guest, n_guest, spacing);
    require(k.guests == species, ALEA_ERR_INVALID_ARGUMENT,
            "FrameworkEnergyGrid::serialize: key guest species differ from the grid's tables");
    std::filesystem::path p(path);
    if (p.has_parent_path()) std::filesystem::create_directories(p.parent_path());
    std::ofstream out(p, std::ios::binary | std::ios::trunc);
    if (!out)
        throw Error(ALEA_ERR_RUNTIME,
                    "FrameworkEnergyGrid::serialize: could not open " + p.string() + " for writing");
    std::string b;
    put(b, kVersion);
    b += key_bytes(k);
    for (int a = 0; a < 3; ++a) put(b, (int32_t)counts[a]);
    put(b, (uint64_t)species.size());
    out.write(b.data(), (std::streamsize)b.size());
    for (size_t i = species.size(); i-- > 0;) {
        std::string t;
        put(t, species[i]);
        put_vec(t, tables[i]);
        out.write(t.data(), (std::streamsize)t.size());
    }
    if (!out)
        throw Error(ALEA_ERR_RUNTIME, "FrameworkEnergyGrid::serialize: write failed for " + p.string());
}

// cacheHit (framework_energy_grid.cc:326-352): false when no file sits at the
// key's content-addressed path; a file there whose version or stored key
// differs is a hard error (never a miss, never a reuse). Reads the header only.
bool grid_cache_hit(const char* dir, const alea_lennard_jones& lj, const alea_particles& fw,
                    const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                    double spacing) {
    const Key key = make_key(lj, fw, lat, guest, n_guest, spacing);
    const std::filesystem::path path = std::filesystem::path(dir) / file_name(key);
    if (!std::filesystem::exists(path)) return false;
    std::ifstream in(path, std::ios::binary);
    if (!in)
        throw Error(ALEA_ERR_RUNTIME, "FrameworkEnergyGrid::cacheHit: could not open " + path.string());
    const uint64_t limit = std::filesystem::file_size(path);
    Reader r{in};
    const uint32_t version = r.get<uint32_t>();
    if (version != kVersion)
        throw Error(ALEA_ERR_RUNTIME, "FrameworkEnergyGrid cache: " + path.string() +
                                          " has format version " + std::to_string(version) +
                                          ", this build expects " + std::to_string(kVersion) +
                                          " -- refusing to reinterpret it. Delete the file (or the "
                                          "cache directory) to force a rebuild.");
    const Key stored = read_key(r, limit);
    if (!in || !(stored == key))
        throw Error(ALEA_ERR_RUNTIME,
                    "FrameworkEnergyGrid cache: " + path.string() +
                        " exists and has a matching content-hash filename, but its stored key does "
                        "not exactly match the current inputs (framework/lattice/force-field/"
                        "spacing) -- this is either a hash collision or a corrupted/foreign cache "
                        "file, and refusing to silently reuse or silently rebuild over it is the "
                        "only safe response. Delete the file if you are sure it is stale.");
    return true;
}

// loadFromCache (framework_energy_grid.cc:354-409)
bool grid_cache_read(const char* dir, const alea_lennard_jones& lj, const alea_particles& fw,
                     const alea_lattice& lat, const uint32_t* guest, uint32_t n_guest,
                     double spacing, int32_t counts[3], std::vector<uint32_t>& species,
                     std::vector<std::vector<double>>& tables) {
    const Key key = make_key(lj, fw, lat, guest, n_guest, spacing);
    const std::filesystem::path path = std::filesystem::path(dir) / file_name(key);
    if (!std::filesystem::exists(path)) return false;
    std::ifstream in(path, std::ios::binary);
    if (!in)
        throw Error(ALEA_ERR_RUNTIME, "FrameworkEnergyGrid::loadFromCache: could not open " + path.string());
    const uint64_t limit = std::filesystem::file_size(path);
    Reader r{in};
    const uint32_t version = r.get<uint32_t>();
    if (version != kVersion)
        throw Error(ALEA_ERR_RUNTIME, "FrameworkEnergyGrid cache: " + path.string() +
                                          " has format version " + std::to_string(version) +
                                          ", this build expects " + std::to_string(kVersion) +
                                          " -- refusing to reinterpret it. Delete the file (or the "
                                          "cache directory) to force a rebuild.");
    const Key stored = read_key(r, limit);
    if (!in)
        throw Error(ALEA_ERR_RUNTIME, "FrameworkEnergyGrid cache: " + path.string() +
                                          " is truncated or corrupt (key read failed)");
    if (!(stored == key))
        throw Error(ALEA_ERR_RUNTIME,
                    "FrameworkEnergyGrid cache: " + path.string() +
                        " exists and has a matching content-hash filename, but its stored key does "
                        "not exactly match the current inputs -- refusing to silently reuse a "
                        "possibly-stale or colliding cache entry. Delete the file if you are sure "
                        "it is stale.");
    for (int a = 0; a < 3; ++a) counts[a] = r.get<int32_t>();
    const uint64_t nt = r.get<uint64_t>();
    std::vector<std::pair<uint32_t, std::vector<double>>> got;
    for (uint64_t i = 0; in && i < nt && i <= limit; ++i) {
        const uint32_t sid = r.get<uint32_t>();
        got.emplace_back(sid, r.get_vec<double>(limit));
    }
    if (!in)
        throw Error(ALEA_ERR_RUNTIME, "FrameworkEnergyGrid cache: " + path.string() +
                                          " is truncated or corrupt (grid data read failed)");
    std::sort(got.begin(), got.end(),
              [](const auto& a, const auto& b) { return a.first < b.first; });
    species.clear();
    tables.clear();
    for (auto& g : got) {
        species.push_back(g.first);
        tables.push_back(std::move(g.second));
    }
    return true;
}

}  // namespace alea
