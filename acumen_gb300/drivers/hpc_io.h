// File and parameter conventions of the reference's driver programs
// (tomography/fits_to_hpc.F90, projections_to_sinogram_hpc.F90, fbp_hpc.F90,
// tv_hpc.F90, tv_hpc_slice.F90), shared by the C++ drivers:
//   $ROOT_CT_DIR/$EXP_CT_NAME/reconstruction/
//     fileinfo_projections.dat  4 floats: nfiles, nimage, n_files_sino, n_files_rec
//     theta.dat                 nfiles floats (degrees)
//     projections{k}.dat        [projection][row][det] floats
//     sinograms{k}.dat          [slice][angle][det] floats, det = nimage+add
//     fbp{k}.dat, fbp_tv{k}.dat [slice][y][x] floats
//   input_parm.txt (8 list-directed lines: nsub, nsub_t, ninner, nouter, ncg,
//   lambda, mu, wpu) and the environment variables of tv_hpc.F90:431-449.
// Raw native-endian FP32, positioned reads and writes (the MPI-IO offsets).
#pragma once
#include <fcntl.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/acumen_gpu.h"

namespace hpc {

struct Fail : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline std::string env(const char* name, bool required = true)
{
    const char* v = std::getenv(name);
    if (!v) {
        if (required) throw Fail(std::string("environment variable ") + name + " is not set");
        return "";
    }
    return v;
}

inline std::string recon_dir()
{
    return env("ROOT_CT_DIR") + "/" + env("EXP_CT_NAME") + "/reconstruction/";
}

inline std::string fnum(const std::string& base, int k) { return base + std::to_string(k) + ".dat"; }

class File {
  public:
    File(const std::string& path, bool write) : path_(path)
    {
        fd_ = ::open(path.c_str(), write ? (O_RDWR | O_CREAT) : O_RDONLY, 0644);
        if (fd_ < 0) throw Fail("cannot open " + path + ": " + std::strerror(errno));
    }
    ~File()
    {
        if (fd_ >= 0) ::close(fd_);
    }
    File(const File&) = delete;
    File& operator=(const File&) = delete;
    // offsets in floats, as the reference's MPI_FILE views of MPI_REAL4
    void read(long long off, float* dst, size_t n) const
    {
        size_t done = 0;
        while (done < n * sizeof(float)) {
            ssize_t r = ::pread(fd_, reinterpret_cast<char*>(dst) + done, n * sizeof(float) - done,
                                (off_t)(off * 4 + (long long)done));
            if (r <= 0) throw Fail("short read from " + path_ + " at float offset " + std::to_string(off));
            done += (size_t)r;
        }
    }
    void write(long long off, const float* src, size_t n) const
    {
        size_t done = 0;
        while (done < n * sizeof(float)) {
            ssize_t r = ::pwrite(fd_, reinterpret_cast<const char*>(src) + done, n * sizeof(float) - done,
                                 (off_t)(off * 4 + (long long)done));
            if (r <= 0) throw Fail("write failed on " + path_);
            done += (size_t)r;
        }
    }

  private:
    std::string path_;
    int fd_ = -1;
};

struct FileInfo {
    int nfiles, nimage, n_files_sino, n_files_rec;
};

// fits_to_hpc.F90:255-267 writes it; tv_hpc.F90:461-477 reads it.
inline FileInfo read_fileinfo(const std::string& dir)
{
    File f(dir + "fileinfo_projections.dat", false);
    float v[4];
    f.read(0, v, 4);
    return FileInfo{(int)v[0], (int)v[1], (int)v[2], (int)v[3]};
}

inline void write_fileinfo(const std::string& dir, const FileInfo& fi)
{
    File f(dir + "fileinfo_projections.dat", true);
    const float v[4] = {(float)fi.nfiles, (float)fi.nimage, (float)fi.n_files_sino, (float)fi.n_files_rec};
    f.write(0, v, 4);
}

inline std::vector<float> read_theta(const std::string& dir, int nfiles)
{
    std::vector<float> t(nfiles);
    File f(dir + "theta.dat", false);
    f.read(0, t.data(), nfiles);
    return t;
}

struct Params {
    int nsub = 1, nsub_t = 1, ninner = 1, nouter = 1, ncg = 1;
    float lambda = 1.0f, mu = 1.0f;
    int wpu = 100;
};

// fbp_hpc.F90:208-217, tv_hpc_slice.F90:419-429: eight list-directed lines
inline Params read_input_parm(const std::string& path)
{
    std::ifstream in(path);
    if (!in) throw Fail("cannot open " + path);
    Params p;
    in >> p.nsub >> p.nsub_t >> p.ninner >> p.nouter >> p.ncg >> p.lambda >> p.mu >> p.wpu;
    if (!in) throw Fail("malformed " + path + " (8 values: nsub nsub_t ninner nouter ncg lambda mu wpu)");
    return p;
}

// tv_hpc.F90:431-449
inline Params env_params()
{
    Params p;
    p.nsub = std::atoi(env("Sub_Sample_Radial").c_str());
    p.nsub_t = std::atoi(env("Sub_Sample_Theta").c_str());
    p.ninner = std::atoi(env("Ninner_Loops").c_str());
    p.nouter = std::atoi(env("Nouter_Loops").c_str());
    p.ncg = std::atoi(env("Opt_ncg").c_str());
    p.lambda = (float)std::atof(env("Opt_lambda").c_str());
    p.mu = (float)std::atof(env("Opt_mu").c_str());
    p.wpu = std::atoi(env("Radon_wpu").c_str());
    return p;
}

// Fortran MINLOC(ABS(theta - target)): first minimum, 1-based
inline int minloc_abs(const std::vector<float>& th, float target)
{
    int best = 1;
    float bv = std::fabs(th[0] - target);
    for (size_t j = 1; j < th.size(); ++j) {
        const float v = std::fabs(th[j] - target);
        if (v < bv) {
            bv = v;
            best = (int)j + 1;
        }
    }
    return best;
}

// Item k (1-based) of a sequence of `count` items split over `nf` files of
// real(count)/real(nf) items each (single-precision arithmetic, as the
// reference): file index j = ceiling(k / r) and the item index inside it.
struct Where {
    int file;        // 1-based
    long long item;  // 0-based position within the file
};
inline Where locate(int k, int count, int nf)
{
    const float r = (float)count / (float)nf;
    const int j = (int)std::ceil((float)k / r);
    const long long item = (long long)k - (long long)std::floor((float)(j - 1) * r) - 1;
    return Where{j, item};
}

inline void check(int rc, acu_ctx* ctx)
{
    if (rc != ACU_OK) throw Fail(std::string("acumen_gpu: ") + acu_last_error(ctx));
}

// ACUMEN_POSITIONS: single-precision sample positions (ACU_OPT_POSITIONS).
// exact (or 1, the default): from the split FP64 angle tables, the mode that
// meets relL2 <= 1e-5 (FBP) and 1e-4 (TV) against FP64 at the benchmark
// sizes; reference (or 0): the reference's own single-precision arithmetic.
inline void apply_positions(acu_ctx* ctx)
{
    const std::string v = env("ACUMEN_POSITIONS", false);
    if (v.empty() || v == "exact" || v == "1") check(acu_set_option(ctx, ACU_OPT_POSITIONS, 1), ctx);
    else if (v == "reference" || v == "0") check(acu_set_option(ctx, ACU_OPT_POSITIONS, 0), ctx);
    else throw Fail("ACUMEN_POSITIONS must be 'reference' (0) or 'exact' (1), got '" + v + "'");
}

// Batches through read -> compute -> write with the file I/O of the next and
// the previous batch overlapping the GPU work of the current one: read(k,
// slot) fills input slot k % 2 on a reader thread, compute(k, slot) turns
// input slot into output slot on the calling thread, write(k, slot) drains
// output slot k % 2 on a writer thread.  A slot is reused only after the
// thread that last used it has been joined.  ACUMEN_PIPELINE=0 runs the three
// in sequence.  An exception on a worker is rethrown on the calling thread.
template <class R, class C, class W>
void pipelined(int nbatches, R read, C compute, W write)
{
    const std::string pv = env("ACUMEN_PIPELINE", false);
    if (pv == "0") {
        for (int k = 0; k < nbatches; ++k) {
            read(k, 0);
            compute(k, 0);
            write(k, 0);
        }
        return;
    }
    std::exception_ptr err_r, err_w;
    auto guard = [](auto fn, std::exception_ptr& e) {
        return [fn, &e](int k, int slot) {
            try {
                fn(k, slot);
            } catch (...) {
                e = std::current_exception();
            }
        };
    };
    auto rd_fn = guard(read, err_r);
    auto wr_fn = guard(write, err_w);
    std::thread rd, wr;
    auto join_all = [&]() {
        if (rd.joinable()) rd.join();
        if (wr.joinable()) wr.join();
    };
    try {
        if (nbatches > 0) rd = std::thread(rd_fn, 0, 0);
        for (int k = 0; k < nbatches; ++k) {
            if (rd.joinable()) rd.join();                         // input k is in slot k % 2
            if (err_r) std::rethrow_exception(err_r);
            if (k + 1 < nbatches) rd = std::thread(rd_fn, k + 1, (k + 1) % 2);
            compute(k, k % 2);                                     // output k into slot k % 2
            if (wr.joinable()) wr.join();                          // output k - 1 written
            if (err_w) std::rethrow_exception(err_w);
            wr = std::thread(wr_fn, k, k % 2);
        }
        join_all();
        if (err_r) std::rethrow_exception(err_r);
        if (err_w) std::rethrow_exception(err_w);
    } catch (...) {
        join_all();
        throw;
    }
}

}  // namespace hpc
