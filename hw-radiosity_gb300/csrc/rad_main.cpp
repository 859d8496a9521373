// ./rad -- drop-in command line of the reference (src/rad.cpp:525-661): same
// options, input, output files and messages, with the shooting loop on the
// GPU through the C ABI.  Extra lines report device statistics.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "rad_gb300.h"

#define KNRM "\x1B[0m"
#define KRED "\x1B[31m"
#define KGRN "\x1B[32m"
#define KMAG "\x1B[35m"
#define KWHT "\x1B[37m"

namespace {

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void usage(const char* argv0, const rad_options& o) {
    fprintf(stderr, "Usage: %s [options] input_file -o output_file\n", argv0);
    fprintf(stderr, "OPTIONS\n");
    fprintf(stderr, "   Debug Options\n");
    fprintf(stderr, "       -debug <integer>        Output intermediate result according debug level.\n");
    fprintf(stderr, "                               " KMAG "Default -debug %d\n\n" KWHT, o.debug);
    fprintf(stderr, "   Radiosity Options\n");
    fprintf(stderr, "       -adapt_area <float>     The threahold of adaptive splitting algorithm.\n");
    fprintf(stderr, "                               " KMAG "Default -area %f\n" KWHT, (double)o.adapt_area);
    fprintf(stderr, "       -sample_area <float>    When the difference of form factor for each vertex is\n");
    fprintf(stderr, "                               greater than delta form factor, it should try to split.\n");
    fprintf(stderr, "                               " KMAG "Default by model-dependent\n" KWHT);
    fprintf(stderr, "       -converge <float>       The radiosity B is the energy per unit area unit B is too small.\n");
    fprintf(stderr, "                               " KMAG "Default -converge %f\n" KWHT, (double)o.converge);
    fprintf(stderr, "       -delta_ff <float>       The difference of delta form factor which is smaller than delta_ff\n");
    fprintf(stderr, "                               will consider as the same.\n");
    fprintf(stderr, "                               " KMAG "Default -delta_ff %f\n" KWHT, (double)o.delta_ff);
    fprintf(stderr, "       -write_cycle <integer>  Write the status of radiosity for each write_cycle iterations.\n");
    fprintf(stderr, "                               " KMAG "Default -write_cycle %d\n" KWHT, o.write_cycle);
    fprintf(stderr, "       -triangle <integer>     The maximum the number of triangles in the model. If you show image\n");
    fprintf(stderr, "                               on WebGL, set -triangle 30000 is the best resolution\n");
    fprintf(stderr, "                               " KMAG "Defulat -triangle %d\n" KWHT, o.triangle_limit);
    fprintf(stderr, "       -light <float>          Adjust the scale of bright light for testing.\n");
    fprintf(stderr, "                               " KMAG "Defulat -light %f\n" KWHT, (double)o.light_scale);
    fprintf(stderr, "       -jobs <integer>         Multithreading OpenMP omp_set_num_threads\n");
    fprintf(stderr, "                               " KMAG "Defulat -jobs %d\n" KWHT, o.jobs);
    fprintf(stderr, "       -parallel_src <integer> The number of light which illuminate other triangles each step\n");
    fprintf(stderr, "                               " KMAG "Defulat -parallel_src %d\n" KWHT, o.parallel_src);
    fprintf(stderr, "   Output Options\n");
    fprintf(stderr, "       -zip                    Compress output file by zip.\n");
    fprintf(stderr, "                               " KMAG "Defulat false\n" KWHT);
    fprintf(stderr, "       -o </<path>/file>       Assign the prefix filename the output file\n");
    fprintf(stderr, "                               " KMAG "Defulat ./test\n" KWHT);
    fprintf(stderr, "       -interactive            Transfer the result into WebGL each write_cycle\n");
    fprintf(stderr, "                               " KMAG "Defulat false\n" KWHT);
    fprintf(stderr, "   GPU Options (extensions)\n");
    fprintf(stderr, "       -device <integer>       CUDA device (default 0)\n");
    fprintf(stderr, "       -fp64                   All-FP64 solver (the reference's float->double build)\n");
    fprintf(stderr, "       -octree_host            Build the octree on the host (default: overlap tests on the GPU)\n");
    fprintf(stderr, "       -init_host              Neighbour links on the host (default: on the GPU)\n");
    fprintf(stderr, "       -autotune               Time both forms of the shooting kernel on the first loops\n");
    fprintf(stderr, "                               and keep the faster (results are the same either way)\n");
    fprintf(stderr, "       -adaptive               Adaptive split variant (config.h = ADAPT + ROLLBACK: serial\n");
    fprintf(stderr, "                               loop, delta-FF split test, no pre-partition)\n");
    fprintf(stderr, "   Headless render of the result (the WebGL viewer's initial view, CUDA rasteriser)\n");
    fprintf(stderr, "       -render <file.ppm>      Write the final result as the viewer shows it\n");
    fprintf(stderr, "       -render_gouraud         Gouraud shading (default: flat, the viewer's default)\n");
    fprintf(stderr, "       -render_size <w> <h>    Image size (default 1024 768, the viewer's canvas)\n");
    fprintf(stderr, "       -render_rot <x> <y>     Rotation about x then y, degrees (default 0 0)\n");
    fprintf(stderr, "   %s -render_fin <in.fin> <out.ppm> [render options]   render an existing result\n", argv0);
}

[[noreturn]] void die(const char* what) {
    fprintf(stderr, "%s\n", what);
    exit(1);
}

void print_log(const rad_scene* s) {
    fputs(rad_scene_log(s, 1), stdout);
    fflush(stdout);
    fputs(rad_scene_log(s, 2), stderr);
}

void check(int rc, const char* what) {
    if (rc != RAD_OK) {
        fprintf(stderr, "[" KRED "ERR" KWHT "] %s: %s\n", what, rad_last_error());
        exit(1);
    }
}

// PrintOut's trailing hooks, src/rad.cpp:224-241
void after_write(const rad_options& o, const std::string& fn) {
    if (o.zip) {
        std::string cmd = "gzip " + fn;
        printf("Compress output file %s .\n", fn.c_str());
        if (system(cmd.c_str())) puts("OK");
        else puts("Failed");
    }
    if (o.interactive) {
        std::string cmd = "cd ./WebGL_demo && ./run.sh ../" + fn + " 2>/dev/null";
        int ret = system(cmd.c_str());
        fprintf(stderr, "WebGL: %s, return %d\n", cmd.c_str(), ret);
    }
}

// headless render of the final result (-render)
const char* g_render = nullptr;
rad_render_options g_ro;

void write_ppm(const char* path, const std::vector<uint8_t>& rgba, int w, int h) {
    FILE* f = fopen(path, "wb");
    if (!f) {
        fprintf(stderr, "[" KRED "ERR" KWHT "] cannot write %s\n", path);
        exit(1);
    }
    fprintf(f, "P6\n%d %d\n255\n", w, h);
    std::vector<uint8_t> rgb((size_t)w * h * 3);
    for (size_t i = 0; i < (size_t)w * h; i++)
        for (int c = 0; c < 3; c++) rgb[i * 3 + c] = rgba[i * 4 + c];
    fwrite(rgb.data(), 1, rgb.size(), f);
    fclose(f);
}

void render_out(const rad_scene* s, int device) {
    if (!g_render) return;
    std::vector<uint8_t> img((size_t)g_ro.width * g_ro.height * 4);
    check(rad_render_scene(s, &g_ro, device, img.data()), "render");
    write_ppm(g_render, img, g_ro.width, g_ro.height);
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Rendered %dx%d image " KMAG "%s\n" KWHT, g_ro.width, g_ro.height, g_render);
}

// render options shared by -render and -render_fin; returns the number of arguments used, 0 if none
int render_opt(int argc, char** argv, int i) {
    auto num = [&](int k, const char* what) -> const char* {
        if (i + k >= argc) die(what);
        return argv[i + k];
    };
    if (!strcmp(argv[i], "-render_gouraud")) { g_ro.shading = 1; return 1; }
    if (!strcmp(argv[i], "-render_size")) {
        if (sscanf(num(1, "RenderSize Error"), "%d", &g_ro.width) != 1 ||
            sscanf(num(2, "RenderSize Error"), "%d", &g_ro.height) != 1)
            die("RenderSize Error");
        return 3;
    }
    if (!strcmp(argv[i], "-render_rot")) {
        if (sscanf(num(1, "RenderRot Error"), "%f", &g_ro.x_rot) != 1 ||
            sscanf(num(2, "RenderRot Error"), "%f", &g_ro.y_rot) != 1)
            die("RenderRot Error");
        return 3;
    }
    if (!strcmp(argv[i], "-render")) { g_render = num(1, "Render path missing"); return 2; }
    return 0;
}

void write_out(const rad_scene* s, const rad_options& o, const char* prefix, int loop) {
    if (rad_scene_write_fin(s, prefix, loop) != RAD_OK) {
        fprintf(stderr, "%s\n", rad_last_error());
        return;
    }
    std::string fn = std::string(prefix) + (loop == 0 ? ".fin" : ("." + std::to_string(loop)));
    after_write(o, fn);
}

// DoRadiosity with serialRadiosity (rad.cpp:491-523 without PRE_PARTITION):
// the adaptive variant updates the host scene in place
int run_adaptive(rad_scene* scene, rad_octree* tree, const rad_options& o, int device, const char* out, double t2) {
    rad_adapt* ad = nullptr;
    check(rad_adapt_create(scene, tree, &o, device, &ad), "device");
    const int W = o.write_cycle;
    long long loop = 1;
    for (;;) {
        long long target = W > 0 ? ((loop + W - 1) / W) * W : loop + (1LL << 40);
        int64_t done = 0;
        int32_t conv = 0;
        int rc = rad_adapt_run(ad, target - loop + 1, &done, &conv);
        if (rc == RAD_ERR_WALK) fprintf(stderr, "[" KRED "WARN" KWHT "] %s\n", rad_last_error());
        else check(rc, "shooting loop");
        print_log(scene);
        long long last = loop + done - 1;
        if (W > 0 && done > 0 && last % W == 0) {
            fprintf(stderr, "[" KGRN "INFO" KWHT "] Loop %lld BEGIN\n", last);
            write_out(scene, o, out, (int)last);
            rad_stats st;
            rad_adapt_stats(ad, &st, nullptr, nullptr, nullptr);
            fprintf(stderr, "[" KGRN "INFO" KWHT "] END Loop. There are %i triangles.\n", st.n_slots);
        }
        loop = last + 1;
        if (conv) {
            if (W > 0 && loop % W == 0) fprintf(stderr, "[" KGRN "INFO" KWHT "] Loop %lld BEGIN\n", loop);
            break;
        }
    }
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Complete in #Iterations %lld\n", loop);
    double a = now();
    write_out(scene, o, out, 0);
    double b = now();
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Store file took " KMAG "%f" KWHT " sec. time.\n", b - a);
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Radiosity Method took " KMAG "%f" KWHT " sec. time.\n", b - t2);
    render_out(scene, device);
    rad_stats st;
    int64_t hp = 0, sp = 0, sm = 0;
    if (rad_adapt_stats(ad, &st, &hp, &sp, &sm) == RAD_OK)
        fprintf(stderr, "[" KGRN "GPU" KWHT "] steps %lld, %d triangles, %lld splits, %lld sample points, "
                "%lld rays (%lld form factors on the host)\n", (long long)st.steps, st.n_slots, (long long)sp,
                (long long)sm, (long long)st.rays, (long long)hp);
    rad_adapt_destroy(ad);
    rad_octree_free(tree);
    rad_scene_free(scene);
    return 0;
}

}  // namespace

int main(int argc, char* argv[]) {
    rad_options o;
    rad_options_default(&o);
    rad_render_options_default(&g_ro);
    int device = 0;
    bool adaptive = false;
    bool autotune = false;
    bool octree_host = false;
    bool init_host = false;
    if (argc < 3) {
        usage(argv[0], o);
        return 1;
    }
    if (!strcmp(argv[1], "-render_fin")) {   // render an existing .fin, no solve
        if (argc < 4) {
            usage(argv[0], o);
            return 1;
        }
        for (int i = 4; i < argc;) {
            int k = render_opt(argc, argv, i);
            if (!k && !strcmp(argv[i], "-device") && i + 1 < argc) {
                device = atoi(argv[i + 1]);
                k = 2;
            }
            if (!k) die("unknown render option");
            i += k;
        }
        std::vector<uint8_t> img((size_t)std::max(g_ro.width, 1) * std::max(g_ro.height, 1) * 4);
        check(rad_render_fin(argv[2], &g_ro, device, img.data()), "render");
        write_ppm(argv[3], img, g_ro.width, g_ro.height);
        return 0;
    }
    static const char* opts[] = {"-debug", "-adapt_area", "-sample_area", "-converge", "-delta_ff",
                                 "-write_cycle", "-zip", "-triangle", "-light", "-o", "-interactive",
                                 "-jobs", "-parallel_src", "-device", "-fp64", "-adaptive", "-autotune",
                                 "-octree_host", "-init_host"};
    const int n_opts = (int)(sizeof opts / sizeof opts[0]);
    const char* in = nullptr;
    const char* out = "./test";
    for (int i = 1; i < argc; i++) {
        if (int k = render_opt(argc, argv, i)) {
            i += k - 1;
            continue;
        }
        int j = 0;
        for (; j < n_opts; j++)
            if (!strcmp(argv[i], opts[j])) break;
        if (j == n_opts) { in = argv[i]; continue; }
        auto need = [&](const char* msg) -> const char* {
            if (i + 1 >= argc) die(msg);
            return argv[++i];
        };
        auto geti = [&](int& dst, const char* msg) { if (sscanf(need(msg), "%d", &dst) != 1) die(msg); };
        auto getf = [&](float& dst, const char* msg) { if (sscanf(need(msg), "%f", &dst) != 1) die(msg); };
        switch (j) {
            case 0: geti(o.debug, "Debug Error"); break;
            case 1: getf(o.adapt_area, "AreaLimit Error"); break;
            case 2: getf(o.sample_area, "SampleArea Error"); break;
            case 3: getf(o.converge, "ConvergeLimit Error"); break;
            case 4: getf(o.delta_ff, "DeltaFFLimit Error"); break;
            case 5: geti(o.write_cycle, "Debug WriteIteration Error"); break;
            case 6: o.zip = 1; break;
            case 7: geti(o.triangle_limit, "TriangleLimit Error"); break;
            case 8: getf(o.light_scale, "LightScale Error"); break;
            case 9: out = need("output prefix missing"); break;
            case 10: o.interactive = 1; break;
            case 11: geti(o.jobs, "Parallel Jobs Error"); break;
            case 12: geti(o.parallel_src, "Parallel Source Error"); break;
            case 13: geti(device, "Device Error"); break;
            case 14: o.precision = 64; break;
            case 15: adaptive = true; break;
            case 16: autotune = true; break;
            case 17: octree_host = true; break;
            case 18: init_host = true; break;
        }
    }
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Input Model " KMAG "%s" KWHT " and Output Prefix " KMAG "%s\n" KWHT,
            in ? in : "(null)", out);
    FILE* probe = in ? fopen(in, "r") : nullptr;
    if (!probe) {
        fprintf(stderr, "File open error::%s\n", argv[2]);
        return 1;
    }
    fclose(probe);

    rad_scene* scene = nullptr;
    rad_octree* tree = nullptr;
    double t0 = now();
    check(rad_scene_load(in, &o, &scene), "scene input");
    print_log(scene);
    // BuildTree with its overlap tests on the GPU (the same leaves and lists as
    // the host build, which -octree_host selects)
    if (octree_host) check(rad_octree_build(scene, o.jobs > 0 ? o.jobs : 0, &tree), "octree");
    else check(rad_octree_build_device(scene, device, &tree), "octree");
    {
        int64_t nodes = 0, lists = 0;
        rad_octree_info(tree, &nodes, &lists, nullptr, nullptr, nullptr);
        fprintf(stderr, "[" KGRN "INFO" KWHT "] 3D-DDA #TreeNode = %lld, #Trilist = %lld\n", (long long)nodes,
                (long long)lists);
    }
    double t1 = now();
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Init took " KMAG "%f" KWHT " sec. time.\n", t1 - t0);

    // DoRadiosity, src/rad.cpp:491-523
    double t2 = now();
    // InitRadiosity; the neighbour links on the GPU unless -init_host
    if (init_host) check(rad_scene_init(scene), "init");
    else check(rad_scene_init_device(scene, device), "init");
    print_log(scene);
    if (adaptive) return run_adaptive(scene, tree, o, device, out, t2);
    check(rad_scene_prepartition(scene), "pre-partition");
    print_log(scene);
    rad_dev* dev = nullptr;
    check(rad_dev_create(scene, tree, &o, device, &dev), "device");
    const int W = o.write_cycle;
    long long loop = 1;
    double ts0 = now();
    for (;;) {
        // shoot loops [loop, target]: up to the next multiple of the write cycle
        long long target = W > 0 ? ((loop + W - 1) / W) * W : loop + (1LL << 40);
        int64_t done = 0;
        int32_t conv = 0;
        int rc;
        if (autotune && loop == 1) {
            int32_t form = 0;
            rc = rad_dev_autotune(dev, 8, std::min<long long>(target - loop + 1, 64), &done, &conv, &form);
            if (rc == RAD_OK || rc == RAD_ERR_WALK)
                fprintf(stderr, "[" KGRN "INFO" KWHT "] Shooting kernel form %d, autotuned over %lld loops\n", form,
                        (long long)done);
        } else {
            rc = rad_dev_run(dev, target - loop + 1, &done, &conv);
        }
        if (rc == RAD_ERR_WALK) fprintf(stderr, "[" KRED "WARN" KWHT "] %s\n", rad_last_error());
        else check(rc, "shooting loop");
        long long last = loop + done - 1;   // last loop that shot
        if (W > 0 && done > 0 && last % W == 0) {
            fprintf(stderr, "[" KGRN "INFO" KWHT "] Loop %lld BEGIN\n", last);
            check(rad_dev_download(dev, scene), "download");
            write_out(scene, o, out, (int)last);
            rad_stats st;
            rad_dev_stats(dev, &st);
            fprintf(stderr, "[" KGRN "INFO" KWHT "] END Loop. There are %i triangles.\n", st.n_slots);
        }
        loop = last + 1;
        if (conv) {
            if (W > 0 && loop % W == 0) fprintf(stderr, "[" KGRN "INFO" KWHT "] Loop %lld BEGIN\n", loop);
            break;
        }
    }
    double ts1 = now();
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Complete in #Iterations %lld\n", loop);
    check(rad_dev_download(dev, scene), "download");
    {
        double a = now();
        write_out(scene, o, out, 0);
        double b = now();
        fprintf(stderr, "[" KGRN "INFO" KWHT "] Store file took " KMAG "%f" KWHT " sec. time.\n", b - a);
    }
    render_out(scene, device);
    double t3 = now();
    fprintf(stderr, "[" KGRN "INFO" KWHT "] Radiosity Method took " KMAG "%f" KWHT " sec. time.\n", t3 - t2);
    rad_stats st;
    if (rad_dev_stats(dev, &st) == RAD_OK) {
        double dt = ts1 - ts0;
        fprintf(stderr,
                "[" KGRN "GPU" KWHT "] steps %lld shots %lld rays %lld in %f s: %.1f shots/s, %.3e rays/s, "
                "precision re-steps %lld, walk-cap hits %lld, device memory %.1f MB, unshot power %.6e\n",
                (long long)st.steps, (long long)st.shots, (long long)st.rays, dt, dt > 0 ? st.shots / dt : 0.0,
                dt > 0 ? st.rays / dt : 0.0, (long long)st.prec_steps, (long long)st.walk_cap_hits,
                st.device_bytes / 1e6, st.unshot_power);
    }
    rad_dev_destroy(dev);
    rad_octree_free(tree);
    rad_scene_free(scene);
    return 0;
}
