// tv_hpc_slice: TV reconstruction of the middle slice only -- the drop-in for
// tomography/tv_hpc_slice.F90:368-588: input_parm.txt, slice nimage/2 of
// sinograms1.dat (the reference reads a single sinogram file, A.2), progress
// line every 10 outer iterations, outputs fbp_tv_slice.dat and
// fbp_sub_slice.dat.
#include "hpc_io.h"

int main()
{
    try {
        using namespace hpc;
        const std::string dir = recon_dir();
        const Params p = read_input_parm(env("ROOT_CT_DIR") + "/" + env("EXP_CT_NAME") + "/input_parm.txt");
        const FileInfo fi = read_fileinfo(dir);
        const int nimagef = fi.nimage, nfiles = fi.nfiles;
        const std::vector<float> f_theta = read_theta(dir, nfiles);
        const int jts = minloc_abs(f_theta, 0.0f), jte = minloc_abs(f_theta, 180.0f);
        const int ntheta = (int)std::floor((float)(jte - jts + 1) / (float)p.nsub_t);
        const int add = nimagef % 2 == 0 ? 1 : 0;
        const int nimage = (int)std::floor((float)(nimagef + add - 1) / (float)p.nsub) + 1;
        std::vector<float> theta(ntheta);
        for (int jy = 1; jy <= ntheta; ++jy) theta[jy - 1] = f_theta[(jy - 1) * p.nsub_t + jts - 1];
        acu_ctx* ctx = nullptr;
        check(acu_ctx_create(&ctx, nimage, ntheta, theta.data(), p.wpu), nullptr);
        apply_positions(ctx);
        check(acu_set_option(ctx, ACU_OPT_VERBOSE, 1), ctx);
        check(acu_set_option(ctx, ACU_OPT_PRINT_EVERY, 10), ctx);
        const int job_id = nimage / 2;                                         // :554
        check(acu_set_option(ctx, 6, job_id), ctx);
        const size_t slab = (size_t)(nimagef + add) * nfiles;
        std::vector<float> sino(slab), f((size_t)ntheta * nimage), tv((size_t)nimage * nimage),
            fbp((size_t)nimage * nimage);
        File fs(fnum(dir + "sinograms", 1), false);
        fs.read((long long)(job_id - 1) * (long long)slab, sino.data(), slab);  // :557-559
        for (int jy = 1; jy <= ntheta; ++jy)
            for (int jx = 1; jx <= nimage; ++jx)
                f[(size_t)(jy - 1) * nimage + jx - 1] =
                    sino[(size_t)((jy - 1) * p.nsub_t + jts - 1) * (nimagef + add) + (jx - 1) * p.nsub];
        check(acu_tvopt(ctx, 1, f.data(), p.ninner, p.nouter, p.ncg, p.lambda, p.mu, tv.data(), fbp.data()), ctx);
        File(dir + "fbp_tv_slice.dat", true).write(0, tv.data(), tv.size());
        File(dir + "fbp_sub_slice.dat", true).write(0, fbp.data(), fbp.size());
        acu_ctx_destroy(ctx);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "tv_hpc_slice: %s\n", e.what());
        return 1;
    }
}
