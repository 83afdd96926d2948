// `lassie input_folder output_folder [-v1|-v2|-v3] [-p double|float]
//        [-engine mixed|fp64] [-root pow|sqrt] [-dump-f64] [-stats]
//        [-controller lassie|bdf] [-rtol R] [-atol A] [-max-order K]`
//
// -controller bdf replaces LASSIE's RKF45/backward-Euler loop with the
// variable-order BDF controller (rtol/atol error control, orders 1..K); the
// atol_vector file, when present, then gives absolute tolerances per species.
//
// Drop-in host for the reference CLI (src/c++/simulator.cu:29-319): the same
// input-folder files and parsing (src/c++/header/Reader.h:23-134), defaults
// and stochastic conversion (Simulation.cuh:263-391, 983-1031), output files
// (Simulation.cuh:451-465, 660-672, 942-971, 1225-1269) and process exit
// codes.  Integration runs on the GPU through the C ABI (lassie_gb300.h).
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <dirent.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "lassie_gb300.h"

namespace {

const char *kStars = "***************************************************************\n";

// ---------------------------------------------------------------- Reader.h

std::vector<std::string> read_lines(const std::string &path) {
    std::vector<std::string> v;
    std::ifstream in(path.c_str());
    std::string line;
    while (std::getline(in, line)) v.push_back(line);
    return v;
}

std::vector<std::string> tab_tokens(const std::string &line) {
    std::vector<std::string> v;
    std::istringstream buf(line);
    for (std::string tok; std::getline(buf, tok, '\t');) v.push_back(tok);
    return v;
}

double parse(const std::string &s) { return std::strtod(s.c_str(), nullptr); }

// readMatrix (Reader.h:104-124); lines without tokens are skipped.
std::vector<std::vector<int>> read_matrix(const std::string &path) {
    std::vector<std::vector<int>> m;
    for (auto &line : read_lines(path)) {
        auto toks = tab_tokens(line);
        if (toks.empty()) continue;
        std::vector<int> row;
        for (auto &t : toks) row.push_back((int)parse(t));
        m.push_back(row);
    }
    return m;
}

std::vector<double> read_by_line(const std::string &path) {
    std::vector<double> v;
    for (auto &line : read_lines(path)) v.push_back(parse(line));
    return v;
}

std::vector<double> read_by_tab(const std::string &path) {
    std::vector<double> v;
    for (auto &line : read_lines(path))
        for (auto &t : tab_tokens(line)) v.push_back(parse(t));
    return v;
}

std::vector<int> read_by_line_int(const std::string &path) {
    std::vector<int> v;
    for (auto &line : read_lines(path)) v.push_back((int)parse(line));
    return v;
}

double read_single(const std::string &path) {
    auto lines = read_lines(path);
    return lines.empty() ? 0.0 : parse(lines[0]);
}

int read_type(const std::string &path) {
    auto lines = read_lines(path);
    const std::string first = lines.empty() ? "" : lines[0];
    if (first == "deterministic" || first == "concentration") return 0;
    if (first == "stochastic" || first == "number") return 1;
    return 2;
}

[[noreturn]] void fail(int code, const std::string &msg) {
    std::printf("\n%s\n", msg.c_str());
    std::printf("%s\n", kStars);
    std::fflush(stdout);
    std::exit(code);
}

bool is_dir(const std::string &p) {
    struct stat sb;
    return stat(p.c_str(), &sb) == 0 && S_ISDIR(sb.st_mode);
}

void write_block_info(const std::string &folder, int sms, const char *type, int n, bool append,
                      int threads_per_cta, int ctas) {
    FILE *fd = std::fopen((folder + "/output/infoBlockThread").c_str(), append ? "a" : "w");
    if (!fd) return;
    if (append) std::fprintf(fd, "\n\n%s \n", type);
    else std::fprintf(fd, "%s \n", type);
    std::fprintf(fd, "Allocating %d threads over %d available streaming multiprocessors\n", n, sms);
    std::fprintf(fd, "Final TPB: %d \n", threads_per_cta);
    std::fprintf(fd, "Number of used blocks: %d \n", ctas);
    std::fprintf(fd, "Total threads spawned: %d \n", threads_per_cta * ctas);
    std::fclose(fd);
}

}  // namespace

// Symbolic right-hand sides (-v2; Simulation.cuh:83-147, printOdes): per
// species the net-stoichiometry terms in reaction order, "+c*k[j]" times
// "*x[i]" once per unit of each reactant's stoichiometry; "dx[i] = 0" when
// there is none.  Fed species print nothing, as in the reference.
static void print_odes(const std::vector<int32_t> &dl, const std::vector<int32_t> &dr, int N,
                       int R, const std::vector<double> &feed) {
    for (int gid = 0; gid < N; gid++) {
        if (feed[gid] != 0) continue;
        std::string s;
        for (int y = 0; y < R; y++) {
            const int c = dr[(size_t)y * N + gid] - dl[(size_t)y * N + gid];
            if (c == 0) continue;
            s += (c > 0 ? "+" : "") + std::to_string(c) + "*k[" + std::to_string(y) + "]";
            for (int i = 0; i < N; i++)
                for (int l = 0; l < dl[(size_t)y * N + i]; l++) s += "*x[" + std::to_string(i) + "]";
        }
        std::printf("dx[%d] = %s\n", gid, s.empty() ? "0" : s.c_str());
    }
}

// Symbolic Jacobian (-v3; Simulation.cuh:149-228, printJac): entry [row][col]
// sums, over the row species' net-stoichiometry terms, the derivative by the
// column species with the reference's conventions -- a reactant of
// stoichiometry 1 gives "+c*k[j]" times the other reactants once each, a
// reactant of stoichiometry a > 1 gives "(c*a)*k[j]" (no explicit "+"),
// x[col] a-1 times and the other reactants once each; a fed column prints 0.
static void print_jacobian(const std::vector<int32_t> &dl, const std::vector<int32_t> &dr, int N,
                           int R, const std::vector<double> &feed) {
    for (int row = 0; row < N; row++) {
        for (int col = 0; col < N; col++) {
            if (feed[col] != 0) {
                std::printf("dx[%d][%d] = 0\n", row, col);
                continue;
            }
            std::string s;
            for (int y = 0; y < R; y++) {
                const int c = dr[(size_t)y * N + row] - dl[(size_t)y * N + row];
                if (c == 0) continue;
                const int a = dl[(size_t)y * N + col];
                if (a < 1) continue;
                std::string others;
                for (int i = 0; i < N; i++)
                    if (i != col && dl[(size_t)y * N + i] > 0)
                        others += "*x[" + std::to_string(i) + "]";
                if (a == 1) {
                    s += (c > 0 ? "+" : "") + std::to_string(c) + "*k[" + std::to_string(y) + "]";
                } else {
                    s += std::to_string(c * a) + "*k[" + std::to_string(y) + "]";
                    for (int l = 0; l < a - 1; l++) s += "*x[" + std::to_string(col) + "]";
                }
                s += others;
            }
            std::printf("dx[%d][%d] = %s\n", row, col, s.empty() ? "0" : s.c_str());
        }
    }
}

int main(int argc, char *argv[]) {
    const auto t_start = std::chrono::steady_clock::now();
    if (argc == 1) {
        std::printf("\nError: the first parameter must be the input folder\n");
        std::printf("\nError: the second parameter must be the output folder\n");
        std::printf("%s\n", kStars);
        return std::exit(-3), 0;
    }
    if (argc == 2) fail(-2, "Eror: the second parameter must be the output folder");

    const std::string path = argv[1];
    DIR *dir = opendir(path.c_str());
    if (!dir) {
        std::printf("\n\n%s\n", kStars);
        fail(-1, "Error: the input folder does not exist");
    }
    std::map<std::string, std::string> files;
    static const char *known[] = {"left_side", "right_side", "c_vector", "t_vector", "M_0",
                                  "cs_vector", "M_feed", "modelkind", "atol_vector", "alphabet",
                                  "be_step", "newton_iter", "newton_tol", "rkf_step",
                                  "stiffness_tol", "volume"};
    for (struct dirent *e; (e = readdir(dir)) != nullptr;) {
        const std::string nm = e->d_name;
        for (const char *k : known)
            if (nm == k) files[nm] = path + "/" + nm;
    }
    closedir(dir);
    // simulator.cu:155-195
    bool to_exit = false;
    const char *mand[][2] = {{"left_side", "there is not left side matrix"},
                             {"right_side", "there is not right side matrix"},
                             {"c_vector", "there is not kinetic constants vector"},
                             {"t_vector", "there is not vector of time instants"},
                             {"M_0", "there is not vector of initial conditions"}};
    for (auto &mm : mand) {
        if (!files.count(mm[0])) {
            std::printf("\n\n%s\n", kStars);
            std::printf("\nError: %s\n", mm[1]);
            std::printf("%s\n", kStars);
            to_exit = true;
        }
    }
    if (to_exit) std::exit(-4);

    const std::string folder = argv[2];
    if (folder[0] == '-' || folder[0] == ' ') {
        std::printf("\n\n%s\n", kStars);
        fail(-2, "Error: the second parameter must be the output folder");
    }
    if (!is_dir(folder)) mkdir(folder.c_str(), 0777);
    if (!is_dir(folder + "/output")) mkdir((folder + "/output").c_str(), 0777);

    int verbose = 0;
    std::string prec = "double";
    std::string engine = "mixed";
    bool dump_f64 = false, want_stats = false, root_sqrt = false;
    std::string controller = "lassie";
    double bdf_rtol = 1e-6, bdf_atol = 1e-9;
    int bdf_max_order = 5;
    for (int i = 3; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "-v1") verbose = 1;
        if (a == "-v2") verbose = 2;
        if (a == "-v3") verbose = 3;
        if (a == "-p") {
            if (i == argc - 1) fail(-5, "Error: you must insert the precison: double or float");
            prec = argv[i + 1];
            if (prec != "double" && prec != "float")
                fail(-6, "Error: the parameter must be double or float");
        }
        if (a == "-engine" && i + 1 < argc) {
            engine = argv[i + 1];
            if (engine != "mixed" && engine != "fp64")
                fail(-6, "Error: the engine must be mixed or fp64");
        }
        if (a == "-root" && i + 1 < argc) {
            const std::string r = argv[i + 1];
            if (r != "pow" && r != "sqrt") fail(-6, "Error: the root must be pow or sqrt");
            root_sqrt = r == "sqrt";
        }
        if (a == "-controller" && i + 1 < argc) {
            controller = argv[i + 1];
            if (controller != "lassie" && controller != "bdf")
                fail(-6, "Error: the controller must be lassie or bdf");
        }
        if (a == "-rtol" && i + 1 < argc) bdf_rtol = std::strtod(argv[i + 1], nullptr);
        if (a == "-atol" && i + 1 < argc) bdf_atol = std::strtod(argv[i + 1], nullptr);
        if (a == "-max-order" && i + 1 < argc) bdf_max_order = std::atoi(argv[i + 1]);
        if (a == "-dump-f64") dump_f64 = true;
        if (a == "-stats") want_stats = true;
    }

    std::printf("\n%s%s", kStars, kStars);
    std::printf("\nLASSIE: A large-scale simulator of mass-action kinetics models\n");

    // ------------------------------------------------- Simulation.cuh:250-391
    auto left = read_matrix(files["left_side"]);
    auto right = read_matrix(files["right_side"]);
    auto c_vector = read_by_line(files["c_vector"]);
    auto t_vector = read_by_line(files["t_vector"]);
    auto M_0 = read_by_tab(files["M_0"]);
    lassie_opts opts;
    lassie_opts_default(&opts);
    opts.precision = engine == "fp64" ? LASSIE_PREC_FP64 : LASSIE_PREC_MIXED;
    // -p float: the reference's single-precision loop (Simulation<float>,
    // simulator.cu:289-294), whatever -engine says
    if (prec == "float") {
        if (controller == "bdf") fail(-6, "Error: -p float runs LASSIE's controller only");
        opts.precision = LASSIE_PREC_FLOAT;
    }
    opts.quarter_root = root_sqrt ? LASSIE_ROOT_SQRT : LASSIE_ROOT_POW;
    if (controller == "bdf") {
        opts.controller = LASSIE_CTRL_BDF;
        opts.rtol = bdf_rtol;
        opts.atol = bdf_atol;
        opts.max_order = bdf_max_order;
    }
    if (files.count("be_step")) opts.be_step = read_single(files["be_step"]);
    if (files.count("rkf_step")) opts.rkf_step = read_single(files["rkf_step"]);
    if (files.count("newton_iter")) opts.newton_iter = (int64_t)(int)read_single(files["newton_iter"]);
    if (files.count("newton_tol")) opts.newton_tol = read_single(files["newton_tol"]);
    if (files.count("stiffness_tol")) opts.stiffness_tol = read_single(files["stiffness_tol"]);
    if (left.empty() || right.empty() || left[0].empty())
        fail(-4, "Error: empty stoichiometry matrix");
    const int R = (int)left.size(), N = (int)left[0].size();
    std::vector<double> atol, feed;
    std::vector<int> cs;
    if (files.count("atol_vector")) atol = read_by_line(files["atol_vector"]);
    else atol.assign(M_0.size(), 1e-12);
    if (files.count("cs_vector")) cs = read_by_line_int(files["cs_vector"]);
    else for (int i = 0; i < (int)M_0.size(); i++) cs.push_back(i);
    if (files.count("M_feed")) feed = read_by_tab(files["M_feed"]);
    else feed.assign(M_0.size(), 0.0);
    const int modelkind = files.count("modelkind") ? read_type(files["modelkind"]) : 0;

    if (verbose) {
        std::printf("\n%s", kStars);
        std::printf("PARAMETERS:\nverbose = true\n");
        std::printf("dt Runge-Kutta-Fehlberg = %g\n", opts.rkf_step);
        std::printf("dt Backward Euler = %g\n", opts.be_step);
        std::printf("Newton's iterations = %lld\n", (long long)opts.newton_iter);
        std::printf("Newton's tollerance = %g\n", opts.newton_tol);
        std::printf("Stiffness tollerance = %g\n", opts.stiffness_tol);
        std::printf("Runge-Kutta-Fehlberg's tollerances = %g\n", atol.empty() ? 0.0 : atol[0]);
        std::printf("Float pointing precision = %s\n", prec.c_str());
        std::printf("Engine = %s\n", engine.c_str());
        if (controller == "bdf")
            std::printf("Controller = BDF (rtol %g, atol %g, orders 1-%d)\n", bdf_rtol, bdf_atol,
                        bdf_max_order);
    }
    if (modelkind == 2) {
        std::printf("\nError: the modelkind can be: deterministic/concentration or stochastic/number\n");
        std::printf("%s\n", kStars);
        std::exit(-7);
    }
    double volume = 1;
    if (modelkind) {
        volume = files.count("volume") ? read_single(files["volume"]) : 0.0;
        if (volume == 0) {
            std::printf("\nError: the modelkind is stochastic/number, but there is not volume file\n");
            std::printf("%s\n", kStars);
            std::exit(-8);
        }
        // Simulation.cuh:983-1031
        const double conv = volume * 6.022e23;
        for (auto &v : M_0) v = v / conv;
        for (auto &v : feed) v = v / conv;
        for (int i = 0; i < (int)c_vector.size(); i++) {
            int nz = 0;
            bool ge2 = false;
            if (i < R)
                for (int j = 0; j < N; j++) {
                    if (left[i][j] > 0) nz++;
                    if (left[i][j] >= 2) ge2 = true;
                }
            if (nz >= 3) {
                std::printf("There are one or more reactions with higher order than the second one\n");
                std::exit(-12);
            }
            if (ge2) c_vector[i] = (c_vector[i] * conv) / 2.0;
            else if (nz > 1) c_vector[i] = c_vector[i] * conv;
        }
    }
    // consistency checks the reference leaves to undefined behaviour
    for (auto &row : left)
        if ((int)row.size() != N) fail(-4, "Error: ragged left side matrix");
    if ((int)right.size() != R) fail(-4, "Error: left and right side matrices differ in size");
    for (auto &row : right)
        if ((int)row.size() != N) fail(-4, "Error: ragged right side matrix");
    if ((int)c_vector.size() < R) fail(-4, "Error: fewer kinetic constants than reactions");
    if ((int)M_0.size() < N) fail(-4, "Error: fewer initial conditions than species");
    if ((int)atol.size() < N) fail(-4, "Error: fewer tolerances than species");
    if ((int)feed.size() < N) fail(-4, "Error: fewer feed values than species");
    for (int c : cs)
        if (c < 0 || c >= N) fail(-4, "Error: cs_vector names a species out of range");

    std::vector<int32_t> dl((size_t)R * N), dr((size_t)R * N);
    for (int j = 0; j < R; j++)
        for (int s = 0; s < N; s++) {
            dl[(size_t)j * N + s] = (int16_t)left[j][s];  // the reference stores shorts
            dr[(size_t)j * N + s] = (int16_t)right[j][s];
        }

    // Simulation.cuh:430-447
    if (verbose > 1) {
        std::printf("\n%sODEs:\n", kStars);
        print_odes(dl, dr, N, R, feed);
        std::printf("%s\n\n", kStars);
    }
    if (verbose > 2) {
        std::printf("\n%sJacobian:\n", kStars);
        print_jacobian(dl, dr, N, R, feed);
        std::printf("%s\n\n", kStars);
    }

    // Simulation.cuh:451-465
    {
        FILE *fd = std::fopen((folder + "/output/SpeciesSampling").c_str(), "w");
        if (!fd) {
            std::perror("Error open output file cs_vector");
            std::exit(-9);
        }
        std::fprintf(fd, "Saving species' dynamics: \n");
        for (int c : cs) std::fprintf(fd, "%d; ", c);
        std::fprintf(fd, "\n");
        std::fclose(fd);
    }

    lassie_model *model = nullptr;
    int rc = lassie_model_create_dense(N, R, dl.data(), dr.data(), &model);
    if (rc) fail(-13, std::string("Error: model: ") + lassie_last_error());
    const int nt = (int)t_vector.size(), ncs = (int)cs.size();
    std::vector<double> out((size_t)nt * ncs, 0.0);
    lassie_stats st{};
    std::vector<int32_t> cs32(cs.begin(), cs.end());
    write_block_info(folder, 0, "ODE", N, false, 512, 1);
    write_block_info(folder, 0, "JAC", N * N, true, 512, 1);
    write_block_info(folder, 0, "DINAM-SUBSPEC", ncs, true, 512, 1);
    if (verbose > 1) std::printf("****Start simulation***\n");
    const auto t_int0 = std::chrono::steady_clock::now();
    // the BDF controller takes per-species tolerances only from atol_vector
    const double *atol_arg =
        (controller == "bdf" && !files.count("atol_vector")) ? nullptr : atol.data();
    rc = lassie_solve(model, c_vector.data(), M_0.data(), feed.data(), atol_arg,
                      t_vector.data(), nt, cs32.data(), ncs, &opts, out.data(), &st);
    const auto t_int1 = std::chrono::steady_clock::now();
    if (rc) {
        std::fprintf(stderr, "Error: %s (%s)\n", lassie_status_string(rc), lassie_last_error());
        lassie_model_destroy(model);
        std::exit(rc == LASSIE_ERR_CUDA ? -13 : -13);
    }
    if (verbose > 1) std::printf("****End simulation***\n");

    // ProgressSimulation (Simulation.cuh:660-672): t/t_max, one line per sample
    {
        FILE *fd = std::fopen((folder + "/output/ProgressSimulation").c_str(), "w");
        if (!fd) {
            std::perror("Error open output file ProgressSimulation");
            std::exit(-11);
        }
        const double t_max = nt > 0 ? t_vector[nt - 1] : 1.0;
        for (int i = 0; i < nt; i++) std::fprintf(fd, "%.4e\n", t_vector[i] / t_max);
        std::fclose(fd);
    }
    // Solution (Simulation.cuh:942-971)
    if (modelkind)
        for (auto &v : out) v = v * (volume * 6.022e23);
    {
        FILE *fd = std::fopen((folder + "/output/Solution").c_str(), "w");
        if (!fd) {
            std::perror("Error open output file Solution");
            std::exit(-11);
        }
        for (int i = 0; i < nt; i++) {
            std::fprintf(fd, "%.4e\t", t_vector[i]);
            for (int j = 0; j < ncs; j++) std::fprintf(fd, "%.4e\t", out[(size_t)i * ncs + j]);
            std::fprintf(fd, "\n");
        }
        std::fclose(fd);
    }
    if (dump_f64) {
        FILE *fd = std::fopen((folder + "/output/Solution.f64").c_str(), "w");
        if (fd) {
            for (int i = 0; i < nt; i++) {
                std::fprintf(fd, "%.17g", t_vector[i]);
                for (int j = 0; j < ncs; j++) std::fprintf(fd, "\t%.17g", out[(size_t)i * ncs + j]);
                std::fprintf(fd, "\n");
            }
            std::fclose(fd);
        }
    }
    const double sim_s = std::chrono::duration<double>(t_int1 - t_int0).count();
    if (want_stats) {
        FILE *fd = std::fopen((folder + "/output/stats.json").c_str(), "w");
        if (fd) {
            std::fprintf(fd,
                         "{\"engine\": \"%s\", \"integration_s\": %.6f, \"outer_iters\": %lld, "
                         "\"rkf_accepts\": %lld, \"rkf_retries\": %lld, \"be_steps\": %lld, "
                         "\"newton_iters\": %lld, \"lu_factorisations\": %lld, "
                         "\"lu_failures\": %lld, \"nan_reverts\": %lld, \"refine_sweeps\": %lld, "
                         "\"t_final\": %.17g, \"dt_be_final\": %.17g, \"controller\": \"%s\", "
                         "\"jac_evals\": %lld, \"rhs_evals\": %lld, \"order_final\": %d}\n",
                         engine.c_str(), sim_s, (long long)st.outer_iters,
                         (long long)st.rkf_accepts, (long long)st.rkf_retries,
                         (long long)st.be_steps, (long long)st.newton_iters,
                         (long long)st.lu_factorisations, (long long)st.lu_failures,
                         (long long)st.nan_reverts, (long long)st.refine_sweeps, st.t_final,
                         st.dt_be_final, controller.c_str(), (long long)st.jac_evals,
                         (long long)st.rhs_evals, (int)st.order_final);
            std::fclose(fd);
        }
    }
    lassie_model_destroy(model);
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    std::printf("\n%s", kStars);
    std::printf("Integration time: %f seconds\n", sim_s);
    std::printf("Total running time: %f seconds\n", total);
    std::printf("%s%s\n", kStars, kStars);
    return 0;
}
