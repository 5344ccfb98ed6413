// Host-side core of the C++ drop-in: the one-rank communicator shim, options, timers, logger, the
// application singleton and the small Vector/Matrix containers user programs touch.
//
// Mirrors the parts user programs call of the reference's src/EllipticForestApp.hpp:39-137,
// src/Options.hpp:27-33 (std::variant<std::string,bool,int,double> options), src/Timer.hpp,
// src/Logger.hpp:31-58, src/MPI.hpp (MPIObject) and src/Vector.hpp / src/Matrix.hpp.  There is no
// MPI, PETSc or p4est: every object lives on one process driving one GPU.
#pragma once

#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
#include <initializer_list>
#include <map>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

#include "../ellipticforest_gb300.h"

#ifndef MPI_COMM_WORLD
// One-rank stand-ins so that reference drivers written against MPI compile unchanged.
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#endif

namespace EllipticForest {

namespace MPI {
using Communicator = MPI_Comm;
constexpr int HEAD_RANK = 0;

// src/MPI.hpp MPIObject: the communicator is accepted and ignored (one rank).
class MPIObject {
public:
    MPIObject() = default;
    explicit MPIObject(Communicator comm) : comm_(comm) {}
    Communicator getComm() const { return comm_; }
    int getRank() const { return 0; }
    int getSize() const { return 1; }

private:
    Communicator comm_ = MPI_COMM_WORLD;
};
}  // namespace MPI

// ---- Options (src/Options.hpp) -------------------------------------------------------------------
class Options {
public:
    using OptionTypes = std::variant<std::string, bool, int, double>;
    std::map<std::string, OptionTypes> optionsMap;

    OptionTypes& operator[](const std::string& key) { return optionsMap[key]; }
    void setOption(const std::string& key, const OptionTypes& value) { optionsMap[key] = value; }
    bool optionExists(const std::string& key) const { return optionsMap.count(key) > 0; }

    // "--key=value" value typing of InputParser.cpp:9-38 / Options::checkValue
    static OptionTypes checkValue(const std::string& v) {
        if (v == "true") return true;
        if (v == "false") return false;
        char* end = nullptr;
        const long iv = std::strtol(v.c_str(), &end, 10);
        if (end && *end == 0 && !v.empty()) return int(iv);
        const double dv = std::strtod(v.c_str(), &end);
        if (end && *end == 0 && !v.empty()) return dv;
        return v;
    }
};

// ---- Timer (src/Timer.hpp): accumulating steady-clock timer ------------------------------------
class Timer {
public:
    using Clock = std::chrono::steady_clock;
    void start() { start_ = Clock::now(); }
    double stop() {
        const double t = std::chrono::duration<double>(Clock::now() - start_).count();
        acc_ += t;
        return t;
    }
    double time() const { return acc_; }
    void restart() { acc_ = 0; }

private:
    double acc_ = 0;
    Clock::time_point start_ = Clock::now();
};

// ---- Logger (src/Logger.hpp:31-58) -------------------------------------------------------------
class Logger {
public:
    bool quiet = false;
    template <class... Args>
    void log(const std::string& message, Args... args) {
        if (quiet) return;
        const std::string s = "[EllipticForest 0] " + message + "\n";
        if constexpr (sizeof...(Args) == 0) {
            std::fputs(s.c_str(), stdout);
        } else {
            // printf-style message with arguments, as the reference's Logger formats it
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wformat-security"
#pragma GCC diagnostic ignored "-Wformat-nonliteral"
            std::printf(s.c_str(), args...);
#pragma GCC diagnostic pop
        }
    }
    template <class... Args>
    void logHead(const std::string& message, Args... args) { log(message, args...); }
};

// ---- Application singleton (src/EllipticForestApp.hpp:39-137) ----------------------------------
class EllipticForestApp {
public:
    Logger logger{};
    Options options{};
    std::map<std::string, Timer> timers{};

    EllipticForestApp() { registry() = this; }
    EllipticForestApp(int* argc, char*** argv) {
        registry() = this;
        timers["app-lifetime"].start();
        if (argc && argv)
            for (int i = 1; i < *argc; ++i) {
                const std::string a = (*argv)[i];
                if (a.rfind("--", 0) != 0) continue;
                const size_t eq = a.find('=');
                if (eq == std::string::npos) continue;
                options.setOption(a.substr(2, eq - 2), Options::checkValue(a.substr(eq + 1)));
            }
    }
    ~EllipticForestApp() {
        if (registry() == this) registry() = nullptr;
    }
    EllipticForestApp(const EllipticForestApp&) = delete;
    EllipticForestApp& operator=(const EllipticForestApp&) = delete;

    static EllipticForestApp& getInstance() {
        if (registry()) return *registry();
        static EllipticForestApp fallback;
        return fallback;
    }

    template <class... Args>
    void log(const std::string& m, Args... a) { logger.log(m, a...); }
    template <class... Args>
    void logHead(const std::string& m, Args... a) { logger.logHead(m, a...); }
    void addTimer(const std::string& name) { timers[name]; }

private:
    static EllipticForestApp*& registry() {
        static EllipticForestApp* p = nullptr;
        return p;
    }
};

// ---- Vector / Matrix (host containers, src/Vector.hpp, src/Matrix.hpp) -------------------------
template <typename T>
class Vector {
public:
    Vector() = default;
    explicit Vector(std::size_t n) : v_(n) {}
    Vector(std::size_t n, T value) : v_(n, value) {}
    Vector(std::initializer_list<T> l) : v_(l) {}
    explicit Vector(std::vector<T> v) : v_(std::move(v)) {}

    std::size_t size() const { return v_.size(); }
    T& operator[](std::size_t i) { return v_[i]; }
    const T& operator[](std::size_t i) const { return v_[i]; }
    std::vector<T>& data() { return v_; }
    const std::vector<T>& data() const { return v_; }
    T* dataPointer() { return v_.data(); }
    const T* dataPointer() const { return v_.data(); }
    std::string& name() { return name_; }
    void append(const Vector& o) { v_.insert(v_.end(), o.v_.begin(), o.v_.end()); }
    Vector getSegment(std::size_t start, std::size_t len) const {
        if (start + len > v_.size()) throw std::out_of_range("[Vector::getSegment] out of range");
        return Vector(std::vector<T>(v_.begin() + start, v_.begin() + start + len));
    }
    void setSegment(std::size_t start, const Vector& o) {
        if (start + o.size() > v_.size()) throw std::out_of_range("[Vector::setSegment] out of range");
        for (std::size_t i = 0; i < o.size(); ++i) v_[start + i] = o[i];
    }

private:
    std::vector<T> v_;
    std::string name_;
};

template <typename T>
Vector<T> concatenate(const std::vector<Vector<T>>& parts) {
    Vector<T> out;
    for (const auto& p : parts) out.append(p);
    return out;
}

template <typename T>
double vectorInfNorm(const Vector<T>& a, const Vector<T>& b) {
    if (a.size() != b.size()) throw std::invalid_argument("[vectorInfNorm] size mismatch");
    double m = 0;
    for (std::size_t i = 0; i < a.size(); ++i) m = std::max(m, std::fabs(double(a[i] - b[i])));
    return m;
}

template <typename T>
class Matrix {
public:
    Matrix() = default;
    Matrix(std::size_t r, std::size_t c, T value = T()) : r_(r), c_(c), v_(r * c, value) {}
    std::size_t nRows() const { return r_; }
    std::size_t nCols() const { return c_; }
    std::size_t nrows() const { return r_; }
    std::size_t ncols() const { return c_; }
    T& operator()(std::size_t i, std::size_t j) { return v_[i * c_ + j]; }  // row-major (Matrix.hpp:711)
    const T& operator()(std::size_t i, std::size_t j) const { return v_[i * c_ + j]; }
    std::vector<T>& data() { return v_; }
    T* dataPointer() { return v_.data(); }

private:
    std::size_t r_ = 0, c_ = 0;
    std::vector<T> v_;
};

// Status check for C-ABI calls made by the drop-in classes: a failure becomes an exception on
// the C++ side of the ABI (as the reference throws for size mismatches).
inline void efCheck(int code, const char* what) {
    if (code != EF_OK) throw std::runtime_error(std::string(what) + ": " + ef_last_error());
}

}  // namespace EllipticForest
