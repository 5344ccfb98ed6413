// Saving and loading a factored tree (no counterpart in the reference, whose operators live only in
// the Node objects of one process): the solve-time operators of every merge node -- T (root solve,
// parent merges), [S | X^{-1}] and the compact H -- and, for FivePointStencil leaves, the sampled
// coefficients and band LU factors, behind a header that records the mesh as its leaf list.  Loading
// rebuilds the mesh and the plan (the index tables, sine bases and eigenvalue tables are derived
// data) and copies the operators back, so a serving process starts warm without re-merging.
//
// File: "EFGBHPS\0", u32 version, i32 solver type, f64 lambda, f64 root box[4], i32 nx, ny, i32 leaf
// count, per leaf (i32 level, i64 ix, i64 iy), payload in node order, u64 FNV-1a hash of the payload.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ef_hps.hpp"

namespace efgb {

namespace {

constexpr char kMagic[8] = {'E', 'F', 'G', 'B', 'H', 'P', 'S', 0};
constexpr uint32_t kVersion = 1;

struct File {
    std::FILE* f = nullptr;
    uint64_t hash = 1469598103934665603ull;  // FNV-1a offset basis
    bool hashing = false;
    ~File() {
        if (f) std::fclose(f);
    }
    void mix(const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) hash = (hash ^ c[i]) * 1099511628211ull;
    }
    void write(const void* p, size_t n) {
        if (std::fwrite(p, 1, n, f) != n) throw std::runtime_error("save: write failed");
        if (hashing) mix(p, n);
    }
    void read(void* p, size_t n) {
        if (std::fread(p, 1, n, f) != n) throw std::invalid_argument("load: file is truncated");
        if (hashing) mix(p, n);
    }
    template <class T>
    void put(const T& v) { write(&v, sizeof(T)); }
    template <class T>
    T get() {
        T v;
        read(&v, sizeof(T));
        return v;
    }
};

void cks(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

template <class T>
void dev_to_file(File& fl, const T* dev, size_t count, std::vector<unsigned char>& buf) {
    buf.resize(count * sizeof(T));
    cks(cudaMemcpy(buf.data(), dev, buf.size(), cudaMemcpyDeviceToHost), "save copy");
    fl.write(buf.data(), buf.size());
}

template <class T>
void file_to_dev(File& fl, T* dev, size_t count, std::vector<unsigned char>& buf) {
    buf.resize(count * sizeof(T));
    fl.read(buf.data(), buf.size());
    cks(cudaMemcpy(dev, buf.data(), buf.size(), cudaMemcpyHostToDevice), "load copy");
}

}  // namespace

// the regions of the payload, in order (the same walk for save and load)
template <class F>
static void walk_payload(Hps& h, F&& region) {
    const Mesh& mesh = h.mesh();
    for (int id = 0; id < h.num_nodes(); ++id) {
        if (mesh.nodes[id].leaf()) continue;
        const NodeDev& nd = h.node(id);
        const size_t s = nd.s;
        region(nd.T, 64 * s * s);
        region(nd.RHS, 48 * s * s);
        region(nd.H, 16 * s * s);
    }
}

void Hps::save(const char* path) const {
    if (!built_) throw std::invalid_argument("save: the FP64 build stage has not run");
    File fl;
    fl.f = std::fopen(path, "wb");
    if (!fl.f) throw std::invalid_argument(std::string("save: cannot open ") + path);
    fl.write(kMagic, 8);
    fl.put(kVersion);
    fl.put(int32_t(solver_type_));
    fl.put(lambda_);
    fl.put(mesh_.xl); fl.put(mesh_.xu); fl.put(mesh_.yl); fl.put(mesh_.yu);
    fl.put(int32_t(mesh_.nx)); fl.put(int32_t(mesh_.ny));
    fl.put(int32_t(mesh_.leaves.size()));
    for (int id : mesh_.leaves) {
        fl.put(int32_t(mesh_.nodes[id].level));
        fl.put(int64_t(mesh_.nodes[id].ix));
        fl.put(int64_t(mesh_.nodes[id].iy));
    }
    fl.hashing = true;
    std::vector<unsigned char> buf;
    // the copies below run on the default stream: finish the tree's own stream first
    cks(cudaStreamSynchronize(st_), "save sync");
    walk_payload(const_cast<Hps&>(*this), [&](double* p, size_t n) { dev_to_file(fl, p, n, buf); });
    if (solver_type_ == SOLVER_FIVE_POINT) {
        const size_t L = mesh_.leaves.size(), nn = size_t(n_) * n_;
        dev_to_file(fl, d_coef_, L * 6 * nn, buf);
        for (size_t k = 0; k < L; ++k) {
            dev_to_file(fl, fp_band_[k], nn * (2 * n_ + 1), buf);
            dev_to_file(fl, fp_bcoef_[k], 4 * size_t(n_), buf);
        }
    }
    fl.hashing = false;
    fl.put(fl.hash);
}

std::unique_ptr<Hps> Hps::load(const char* path) {
    File fl;
    fl.f = std::fopen(path, "rb");
    if (!fl.f) throw std::invalid_argument(std::string("load: cannot open ") + path);
    char magic[8];
    fl.read(magic, 8);
    if (std::memcmp(magic, kMagic, 8) != 0) throw std::invalid_argument("load: not a saved HPS tree");
    if (fl.get<uint32_t>() != kVersion) throw std::invalid_argument("load: unsupported file version");
    const int type = fl.get<int32_t>();
    const double lambda = fl.get<double>();
    const double xl = fl.get<double>(), xu = fl.get<double>(), yl = fl.get<double>(), yu = fl.get<double>();
    const int nx = fl.get<int32_t>(), ny = fl.get<int32_t>();
    const int nl = fl.get<int32_t>();
    if (nl <= 0 || nl > (1 << 28)) throw std::invalid_argument("load: bad leaf count");
    std::vector<Quad> leaves(nl);
    for (auto& q : leaves) {
        q.level = fl.get<int32_t>();
        q.ix = fl.get<int64_t>();
        q.iy = fl.get<int64_t>();
    }
    const Mesh mesh = Mesh::from_leaves(xl, xu, yl, yu, nx, ny, leaves);
    if (int(mesh.leaves.size()) != nl) throw std::invalid_argument("load: the leaf list is not a balanced quadtree");
    auto h = std::make_unique<Hps>(mesh, type, lambda, false);
    fl.hashing = true;
    std::vector<unsigned char> buf;
    walk_payload(*h, [&](double* p, size_t n) { file_to_dev(fl, p, n, buf); });
    if (type == SOLVER_FIVE_POINT) {
        const size_t L = h->mesh_.leaves.size(), nn = size_t(h->n_) * h->n_;
        file_to_dev(fl, h->d_coef_, L * 6 * nn, buf);
        for (size_t k = 0; k < L; ++k) {
            file_to_dev(fl, h->fp_band_[k], nn * (2 * h->n_ + 1), buf);
            file_to_dev(fl, h->fp_bcoef_[k], 4 * size_t(h->n_), buf);
        }
        h->coef_set_ = true;
    }
    fl.hashing = false;
    const uint64_t want = fl.hash;
    if (fl.get<uint64_t>() != want) throw std::invalid_argument("load: checksum mismatch (corrupted file)");
    cks(cudaDeviceSynchronize(), "load sync");  // the default-stream uploads are done before any kernel reads them
    h->built_ = true;
    return h;
}

}  // namespace efgb
