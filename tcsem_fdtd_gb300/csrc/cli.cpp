// tcsem_fdtd: drop-in replacement of the reference executable TCSEM_FDTD_GPU.
// Reads FDTD_setup.in, Cond.bin, Receiver.in and Transmitter.in from the
// working directory (or the directory given as the first argument), runs every
// transmitter and writes Tx<k>.bout and testwaveform.dat like main.cu:58-324.
// Options: --fp64 (double-precision build mode), --device N, --fix-dual-bipole,
// --batch (all transmitters advanced together as one device batch; --persistent: its
// persistent schedule, one launch per block of steps), --padded-plane /
// --smooth-plane (air field continued on a power-of-two / 5-smooth plane with tapered
// edges; not the reference's arithmetic).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tcsem.h"

int main(int argc, char **argv) {
    std::string dir = ".";
    tcsem_opts o;
    tcsem_default_opts(&o);
    bool batch = false;
    for (int a = 1; a < argc; a++) {
        if (!std::strcmp(argv[a], "--fp64")) o.precision = TCSEM_FP64;
        else if (!std::strcmp(argv[a], "--batch")) batch = true;
        else if (!std::strcmp(argv[a], "--persistent")) o.persistent_batch = 1;
        else if (!std::strcmp(argv[a], "--fix-dual-bipole")) o.fix_dual_bipole = 1;
        else if (!std::strcmp(argv[a], "--padded-plane")) o.padded_plane = 1;
        else if (!std::strcmp(argv[a], "--smooth-plane")) o.padded_plane = 2;
        else if (!std::strcmp(argv[a], "--device") && a + 1 < argc) o.device = std::atoi(argv[++a]);
        else if (argv[a][0] != '-') dir = argv[a];
        else {
            std::fprintf(stderr, "usage: tcsem_fdtd [dir] [--fp64] [--device N] [--fix-dual-bipole] "
                                 "[--batch [--persistent]] [--padded-plane | --smooth-plane]\n");
            return 2;
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    tcsem_sim_t *sim = nullptr;
    tcsem_status st = tcsem_open_dir(dir.c_str(), &o, &sim);
    if (st != TCSEM_OK) {
        std::fprintf(stderr, "Error: unable to load the setup or model (%d): %s\n", (int)st, tcsem_open_error());
        return 1;
    }
    std::printf("The model is initialized successfully!\n");
    tcsem_info info;
    tcsem_get_info(sim, &info);
    std::printf("time iteration =%ld\n", info.nsteps);
    {  // testwaveform.dat, SourceWave.cpp:60-71
        int nsrc = 0;
        tcsem_get_waveform(sim, &nsrc, nullptr, nullptr, nullptr);
        std::vector<double> t(2 * nsrc + 1), dt(2 * nsrc + 1), w(2 * nsrc + 1);
        tcsem_get_waveform(sim, &nsrc, t.data(), dt.data(), w.data());
        std::string p = dir + "/testwaveform.dat";
        FILE *f = std::fopen(p.c_str(), "wb");
        if (f) {
            std::fwrite(&nsrc, sizeof(int), 1, f);
            std::fwrite(t.data(), sizeof(double), t.size(), f);
            std::fwrite(dt.data(), sizeof(double), dt.size(), f);
            std::fwrite(w.data(), sizeof(double), w.size(), f);
            std::fclose(f);
        }
    }
    auto tg = std::chrono::steady_clock::now();
    int rc = 0;
    if (batch) {  // every transmitter as one slot of a device batch
        tcsem_close(sim);
        tcsem_batch_t *b = nullptr;
        if (tcsem_batch_create(&o, 0, &b) != TCSEM_OK) {
            std::fprintf(stderr, "Error: %s\n", tcsem_batch_error(nullptr));
            return 1;
        }
        std::vector<int> slots(info.NTx, -1);
        for (int itx = 0; itx < info.NTx; itx++) {
            std::printf("start to model the EM field generated by Tx %d\n", itx + 1);
            if (tcsem_batch_add(b, dir.c_str(), itx, &slots[itx]) != TCSEM_OK) {
                std::fprintf(stderr, "Error in transmitter %d: %s\n", itx + 1, tcsem_batch_error(b));
                slots[itx] = -1;
                rc = 1;
            }
        }
        int running = 0;
        do {
            if (tcsem_batch_advance(b, 1024) != TCSEM_OK) {
                std::fprintf(stderr, "Error: %s\n", tcsem_batch_error(b));
                rc = 1;
                break;
            }
            tcsem_batch_stats(b, nullptr, &running, nullptr);
        } while (running > 0);
        int nd = 0;
        tcsem_batch_poll(b, nullptr, 0, &nd);
        for (int itx = 0; itx < info.NTx; itx++) {
            if (slots[itx] < 0) continue;
            char name[64];
            std::snprintf(name, sizeof name, "/Tx%d.bout", itx + 1);
            if (tcsem_batch_write_bout(b, slots[itx], (dir + name).c_str()) != TCSEM_OK) {
                std::fprintf(stderr, "Error writing %s: %s\n", name + 1, tcsem_batch_error(b));
                rc = 1;
            }
            std::printf("end of time iteration for Tx %d\n", itx + 1);
        }
        tcsem_batch_destroy(b);
        auto t1 = std::chrono::steady_clock::now();
        std::printf("FDTD modleing completed, runtime=%8.1f sec.\n", std::chrono::duration<double>(t1 - t0).count());
        std::printf("Pure GPU runtime=%8.1f sec.\n", std::chrono::duration<double>(t1 - tg).count());
        return rc;
    }
    // traces of one transmitter fit in NRx*NComp*Nt doubles
    std::vector<double> traces((size_t)info.NRx * info.NComp * info.Nt);
    for (int itx = 0; itx < info.NTx; itx++) {
        std::printf("start to model the EM field generated by Tx %d\n", itx + 1);
        st = tcsem_run(sim, itx, traces.data());
        if (st != TCSEM_OK) {
            std::fprintf(stderr, "Error in transmitter %d (%d): %s\n", itx + 1, (int)st, tcsem_last_error(sim));
            rc = 1;
            continue;
        }
        char name[64];
        std::snprintf(name, sizeof name, "/Tx%d.bout", itx + 1);
        st = tcsem_write_bout(sim, itx, traces.data(), (dir + name).c_str());
        if (st != TCSEM_OK) {
            std::fprintf(stderr, "Error writing %s: %s\n", name + 1, tcsem_last_error(sim));
            rc = 1;
        }
        std::printf("end of time iteration for Tx %d\n", itx + 1);
    }
    auto t1 = std::chrono::steady_clock::now();
    std::printf("FDTD modleing completed, runtime=%8.1f sec.\n", std::chrono::duration<double>(t1 - t0).count());
    std::printf("Pure GPU runtime=%8.1f sec.\n", std::chrono::duration<double>(t1 - tg).count());
    tcsem_close(sim);
    return rc;
}
