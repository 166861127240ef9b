// fbp_hpc: filtered backprojection of every slice -- the drop-in for
// tomography/fbp_hpc.F90:156-425.  Reads input_parm.txt (only wpu matters:
// the reference forces nsub = nsub_t = 1, :280-281), the 4-float fileinfo,
// theta.dat and sinograms{k}.dat, and writes fbp{k}.dat.  The parameters are
// not written back into the fileinfo (the reference's offsets 2-9 overwrite
// clash with the 4-float layout the other programs read).  Slices are
// reconstructed in batches of ACUMEN_BATCH (default 256) on the GPU, with the
// file reads of the next batch and the writes of the previous one overlapping
// the current batch's reconstruction (ACUMEN_PIPELINE=0: in sequence).
#include <chrono>
#include <memory>

#include "hpc_io.h"

int main()
{
    try {
        using namespace hpc;
        const std::string dir = recon_dir();
        const std::string parm = env("ROOT_CT_DIR") + "/" + env("EXP_CT_NAME") + "/input_parm.txt";
        std::printf(" Updating from file: %s\n", parm.c_str());
        const Params p = read_input_parm(parm);
        const auto t0 = std::chrono::steady_clock::now();
        const FileInfo fi = read_fileinfo(dir);
        const int nimagef = fi.nimage, nfiles = fi.nfiles;
        const std::vector<float> f_theta = read_theta(dir, nfiles);
        const int jts = minloc_abs(f_theta, 0.0f), jte = minloc_abs(f_theta, 180.0f);
        const int ntheta = jte - jts + 1;                                     // :324
        const int add = nimagef % 2 == 0 ? 1 : 0;
        const int nimage = nimagef + add;                                     // :329
        std::vector<float> theta(f_theta.begin() + (jts - 1), f_theta.begin() + (jts - 1) + ntheta);
        std::printf(" Reconstruction with Resolution: %d with %d projections\n", nimage, ntheta);
        acu_ctx* ctx = nullptr;
        check(acu_ctx_create(&ctx, nimage, ntheta, theta.data(), p.wpu), nullptr);
        apply_positions(ctx);
        std::vector<std::unique_ptr<File>> fsino, frec;
        for (int k = 1; k <= fi.n_files_sino; ++k) fsino.emplace_back(new File(fnum(dir + "sinograms", k), false));
        for (int k = 1; k <= fi.n_files_rec; ++k) frec.emplace_back(new File(fnum(dir + "fbp", k), true));
        const int batch = std::max(1, std::atoi((std::getenv("ACUMEN_BATCH") ? std::getenv("ACUMEN_BATCH") : "256")));
        const size_t slab = (size_t)nimage * nfiles;
        // two input and two output buffers: the next batch is read and the
        // previous one written while the GPU reconstructs the current one
        std::vector<float> sino[2], f[2], img[2];
        for (int k = 0; k < 2; ++k) {
            sino[k].resize(slab);
            f[k].resize((size_t)batch * ntheta * nimage);
            img[k].resize((size_t)batch * nimage * nimage);
        }
        const int nb = (nimagef + batch - 1) / batch;
        auto count = [&](int k) { return std::min(batch, nimagef - k * batch); };
        pipelined(
            nb,
            [&](int k, int slot) {
                for (int b = 0; b < count(k); ++b) {
                    const Where w = locate(k * batch + b + 1, nimagef, fi.n_files_sino);   // :383-392
                    fsino[w.file - 1]->read(w.item * (long long)slab, sino[slot].data(), slab);
                    std::memcpy(f[slot].data() + (size_t)b * ntheta * nimage,
                                sino[slot].data() + (size_t)(jts - 1) * nimage, sizeof(float) * (size_t)ntheta * nimage);
                }
            },
            [&](int k, int slot) { check(acu_iradon(ctx, count(k), f[slot].data(), img[slot].data()), ctx); },  // :394
            [&](int k, int slot) {
                for (int b = 0; b < count(k); ++b) {
                    const Where w = locate(k * batch + b + 1, nimagef, fi.n_files_rec);    // :396-398
                    frec[w.file - 1]->write(w.item * (long long)nimage * nimage,
                                            img[slot].data() + (size_t)b * nimage * nimage, (size_t)nimage * nimage);
                }
            });
        acu_ctx_destroy(ctx);
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf(" Total Compute time: %g\n", secs);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "fbp_hpc: %s\n", e.what());
        return 1;
    }
}
