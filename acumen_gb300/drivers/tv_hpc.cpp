// tv_hpc: split-Bregman TV reconstruction of every slice -- the drop-in for
// tomography/tv_hpc.F90:392-653.  Same environment variables, fileinfo,
// theta.dat, sinograms{k}.dat input and fbp{k}.dat / fbp_tv{k}.dat (or
// fbp_sub / fbp_sub_tv when sub-sampling) outputs.  The MPI master/worker
// queue over slices (:583-631) is replaced by batches of slices solved
// together on the GPU (ACUMEN_BATCH slices per batch, default 256).
#include <chrono>

#include "hpc_io.h"

int main()
{
    try {
        using namespace hpc;
        const std::string dir = recon_dir();
        const Params p = env_params();
        std::printf(" Running: %s\n  Itr: %d\n  Lambda: %g\n  Mu: %g\n", env("EXP_CT_NAME").c_str(), p.nouter,
                    p.lambda, p.mu);
        const auto t0 = std::chrono::steady_clock::now();
        const FileInfo fi = read_fileinfo(dir);
        const int nimagef = fi.nimage, nfiles = fi.nfiles;
        const std::vector<float> f_theta = read_theta(dir, nfiles);
        const int jts = minloc_abs(f_theta, 0.0f), jte = minloc_abs(f_theta, 180.0f);
        const int ntheta = (int)std::floor((float)(jte - jts + 1) / (float)p.nsub_t);   // :550
        const int add = nimagef % 2 == 0 ? 1 : 0;
        const int nimage = (int)std::floor((float)(nimagef + add - 1) / (float)p.nsub) + 1;  // :555
        std::vector<float> theta(ntheta);
        for (int jy = 1; jy <= ntheta; ++jy) theta[jy - 1] = f_theta[(jy - 1) * p.nsub_t + jts - 1];
        if ((nimage - 1) * p.nsub != nimagef + add - 1) std::printf(" Warning:  nsub must evenly sub-divide\n");
        std::printf(" Reconstruction with Resolution: %d with %d projections\n", nimage, ntheta);
        acu_ctx* ctx = nullptr;
        check(acu_ctx_create(&ctx, nimage, ntheta, theta.data(), p.wpu), nullptr);
        apply_positions(ctx);
        check(acu_set_option(ctx, ACU_OPT_VERBOSE, 1), ctx);
        check(acu_set_option(ctx, ACU_OPT_PRINT_EVERY, 50), ctx);
        const bool sub = p.nsub + p.nsub_t != 2;
        std::vector<std::unique_ptr<File>> fsino, frec, frec_tv;
        for (int k = 1; k <= fi.n_files_sino; ++k) fsino.emplace_back(new File(fnum(dir + "sinograms", k), false));
        for (int k = 1; k <= fi.n_files_rec; ++k) {
            frec.emplace_back(new File(fnum(dir + (sub ? "fbp_sub" : "fbp"), k), true));
            frec_tv.emplace_back(new File(fnum(dir + (sub ? "fbp_sub_tv" : "fbp_tv"), k), true));
        }
        const int batch = std::max(1, std::atoi((std::getenv("ACUMEN_BATCH") ? std::getenv("ACUMEN_BATCH") : "256")));
        const size_t slab = (size_t)(nimagef + add) * nfiles;
        std::vector<float> sino(slab), f((size_t)batch * ntheta * nimage), tv((size_t)batch * nimage * nimage),
            fbp((size_t)batch * nimage * nimage);
        for (int s0 = 1; s0 <= nimagef; s0 += batch) {
            const int B = std::min(batch, nimagef - s0 + 1);
            for (int b = 0; b < B; ++b) {
                const Where w = locate(s0 + b, nimagef, fi.n_files_sino);      // :609-612
                fsino[w.file - 1]->read(w.item * (long long)slab, sino.data(), slab);
                float* fb = f.data() + (size_t)b * ntheta * nimage;
                for (int jy = 1; jy <= ntheta; ++jy)                           // :614-618
                    for (int jx = 1; jx <= nimage; ++jx)
                        fb[(size_t)(jy - 1) * nimage + jx - 1] =
                            sino[(size_t)((jy - 1) * p.nsub_t + jts - 1) * (nimagef + add) + (jx - 1) * p.nsub];
            }
            check(acu_set_option(ctx, 6, s0), ctx);
            check(acu_tvopt(ctx, B, f.data(), p.ninner, p.nouter, p.ncg, p.lambda, p.mu, tv.data(), fbp.data()), ctx);
            for (int b = 0; b < B; ++b) {                                      // :622-626
                const Where w = locate(s0 + b, nimagef, fi.n_files_rec);
                const long long off = w.item * (long long)nimage * nimage;
                frec[w.file - 1]->write(off, fbp.data() + (size_t)b * nimage * nimage, (size_t)nimage * nimage);
                frec_tv[w.file - 1]->write(off, tv.data() + (size_t)b * nimage * nimage, (size_t)nimage * nimage);
            }
        }
        acu_ctx_destroy(ctx);
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf(" Total Compute time: %g\n", secs);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "tv_hpc: %s\n", e.what());
        return 1;
    }
}
