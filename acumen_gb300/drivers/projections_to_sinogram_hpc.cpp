// projections_to_sinogram_hpc: the drop-in for
// tomography/projections_to_sinogram_hpc.F90.  Reads the fileinfo, theta.dat
// and the normalised projections{k}.dat (nfiles square nimage x nimage
// projections), finds the 0 and 180-degree projections, registers the
// rotation axis (ACUMEN_REGISTRATION = pattern (default, the reference's
// search) or xcorr), applies the 27-point median and the rotation / shift
// correction, and writes slice-major sinograms{k}.dat.  The reference's
// per-row MPI_FILE_WRITE_AT calls (:481-487) become one write per slice.
#include <chrono>

#include "hpc_io.h"

int main()
{
    try {
        using namespace hpc;
        const std::string dir = recon_dir();
        const auto t0 = std::chrono::steady_clock::now();
        const FileInfo fi = read_fileinfo(dir);
        const int nfiles = fi.nfiles, nimage = fi.nimage;
        std::printf(" Working on: %s  With number of projections: %d\n", env("EXP_CT_NAME").c_str(), nfiles);
        const std::vector<float> f_theta = read_theta(dir, nfiles);
        const int add = nimage % 2 == 0 ? 1 : 0;
        const size_t npix = (size_t)nimage * nimage;
        std::vector<float> proj(npix * nfiles);
        std::vector<std::unique_ptr<File>> fpro, fsino;
        for (int k = 1; k <= fi.n_files_sino; ++k) {
            fpro.emplace_back(new File(fnum(dir + "projections", k), false));
            fsino.emplace_back(new File(fnum(dir + "sinograms", k), true));
        }
        for (int job = 1; job <= nfiles; ++job) {                             // :397-400
            const Where w = locate(job, nfiles, fi.n_files_sino);
            fpro[w.file - 1]->read(w.item * (long long)npix, proj.data() + (size_t)(job - 1) * npix, npix);
        }
        const char* reg = std::getenv("ACUMEN_REGISTRATION");
        const int method = (reg && std::string(reg) == "xcorr") ? 1 : 0;
        acu_ctx* ctx = nullptr;
        check(acu_ctx_create(&ctx, 0, 0, nullptr, 0), nullptr);
        std::vector<float> sino((size_t)nimage * nfiles * (nimage + add));
        float best_theta = 0.f, best_shift = 0.f;
        check(acu_proj_to_sino(ctx, nfiles, nimage, nimage, proj.data(), f_theta.data(), method, sino.data(),
                               &best_theta, &best_shift),
              ctx);
        std::printf(" Best theta: %15.7E  Best shift: %15.7E\n", best_theta, best_shift);   // :365-367
        const size_t slab = (size_t)nfiles * (nimage + add);
        for (int jy = 1; jy <= nimage; ++jy) {                                // :481-487
            const Where w = locate(jy, nimage, fi.n_files_sino);
            fsino[w.file - 1]->write(w.item * (long long)slab, sino.data() + (size_t)(jy - 1) * slab, slab);
        }
        acu_ctx_destroy(ctx);
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf(" Total Compute time: %g\n", secs);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "projections_to_sinogram_hpc: %s\n", e.what());
        return 1;
    }
}
