// cmp-gb300 / crs-gb300: drop-in command lines for the reference's cmp-* and crs-*
// programs (CMP/OpenMP/src/main.cpp:51-278, CRS/OpenMP/src/main.cpp:59-379).
//
// Same flags and the same parsing rules as the reference parser
// (CMP/OpenMP/src/parser.cpp:44-103): arguments come in "-flag value" pairs, an
// unknown flag or "-h" prints the help and exits with status 1, a missing required
// flag does the same, and a repeated flag keeps its first value.  CMP numbers are
// read with stof, CRS numbers with stod.  Outputs go to the current directory under
// the reference's names; with -v 2 the INFO line reports the execution time and the
// reference's semblance-trace rate.  Extra flags, all optional:
//   -mode plain|batched   search form (default plain: the reference's FP32 order)
//   -store f16|bf16|f32   trace storage of the batched form (default f16)
//   -d N                  CUDA device (default 0)
// CRS also accepts -azimuth (degrees), which does not change the search.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "semb_gb300.h"

#ifndef SEMB_CLI_METHOD
#define SEMB_CLI_METHOD SEMB_CMP
#endif

namespace {

std::map<std::string, std::string> g_flags;   // flag -> help
std::map<std::string, std::string> g_raw;      // flag -> value (first occurrence)
std::string g_prog;
int g_verbosity = 0;                            // 0 FAIL, 1 WARNING, 2 INFO, 3 DEBUG

void print_help() {
  std::printf("Usage: %s [options]\nOptions: \n", g_prog.c_str());
  for (auto& kv : g_flags) std::printf("  %s: %s\n", kv.first.c_str(), kv.second.c_str());
}

[[noreturn]] void die_help() {
  print_help();
  std::exit(EXIT_FAILURE);
}

[[noreturn]] void die(const char* where, int line, const std::string& msg) {
  std::fprintf(stderr, "[FAIL]: %s:%d: %s\n", where, line, msg.c_str());
  std::exit(EXIT_FAILURE);
}

#define FAIL(msg) die(__FILE__, __LINE__, msg)

void info(const char* where, int line, const std::string& msg) {
  if (g_verbosity >= 2) std::printf("[INFO]: %s:%d: %s\n", where, line, msg.c_str());
}

void parse(int argc, const char** argv) {
  g_prog = argv[0];
  if (!(argc % 2) || argc == 1) die_help();
  for (int i = 1; i < argc; i += 2) {
    if (!g_flags.count(argv[i]) || !std::strcmp(argv[i], "-h") || !std::strcmp(argv[i + 1], "-h")) die_help();
    g_raw.insert({argv[i], argv[i + 1]});
  }
}

std::string get(const std::string& k, bool required, const char* dflt = "0") {
  auto it = g_raw.find(k);
  if (it != g_raw.end()) return it->second;
  if (required) die_help();
  return dflt;
}

void check(int rc, const char* what) {
  if (rc != SEMB_OK) FAIL(std::string(what) + ": " + semb_strerror(rc) + ": " + semb_last_error());
}

}  // namespace

int main(int argc, const char** argv) {
  const int method = SEMB_CLI_METHOD;
  if (method == SEMB_CRS) {
    g_flags = {{"-a0", "A0 constant"},   {"-a1", "A1 constant"},   {"-na", "NA constant"},
               {"-b0", "B0 constant"},   {"-b1", "B1 constant"},   {"-nb", "NB constant"},
               {"-c0", "C0 constant"},   {"-c1", "C1 constant"},   {"-nc", "NC constant"},
               {"-aph", "APH constant"}, {"-apm", "APM constant"}, {"-azimuth", "Azimuth angle"},
               {"-tau", "Tau constant"}, {"-i", "Data path"},      {"-v", "Verbosity Level 0-3"}};
  } else {
    g_flags = {{"-c0", "C0 constant"}, {"-c1", "C1 constant"},   {"-nc", "NC constant"},
               {"-aph", "APH constant"}, {"-tau", "Tau constant"}, {"-i", "Data path"},
               {"-v", "Verbosity Level 0-3"}};
  }
  g_flags["-mode"] = "Search form: plain (default) or batched";
  g_flags["-store"] = "Trace storage of the batched form: f16 (default), bf16 or f32";
  g_flags["-d"] = "CUDA device";
  if (method == SEMB_CRS) g_flags["-dm"] = "Midpoint displacement: abs (default, as the reference) or signed (along -azimuth)";
  if (method == SEMB_CRS) g_flags["-ngen"] = "Generations of the CRS-DE search (differential evolution; 0: grid search)";
  g_flags["-attrs"] = "1: also write <method>.aperture.su and, batched, <method>.coher2.su and <method>.err64.su";
  parse(argc, argv);

  semb_params p;
  semb_params_init(&p, method);
  try {
    if (method == SEMB_CMP) {
      p.c0 = std::stof(get("-c0", true));
      p.c1 = std::stof(get("-c1", true));
      p.tau = std::stof(get("-tau", true));
    } else {
      p.a0 = std::stod(get("-a0", true));
      p.a1 = std::stod(get("-a1", true));
      p.b0 = std::stod(get("-b0", true));
      p.b1 = std::stod(get("-b1", true));
      p.c0 = std::stod(get("-c0", true));
      p.c1 = std::stod(get("-c1", true));
      p.tau = std::stod(get("-tau", true));
      p.na = std::stoi(get("-na", true));
      p.nb = std::stoi(get("-nb", true));
      p.apm = std::stoi(get("-apm", true));
      p.azimuth = std::stod(get("-azimuth", false));
    }
    p.nc = std::stoi(get("-nc", true));
    p.aph = std::stoi(get("-aph", true));
    g_verbosity = std::stoi(get("-v", false));
  } catch (const std::exception& e) {
    FAIL(std::string("bad numeric argument: ") + e.what());
  }
  const std::string path = get("-i", true);
  const std::string mode = get("-mode", false, "plain");
  const std::string store = get("-store", false, "f16");
  const int device = std::atoi(get("-d", false, "0").c_str());
  if (mode == "plain") p.mode = SEMB_PLAIN_F32;
  else if (mode == "batched") p.mode = SEMB_BATCHED;
  else die_help();
  if (store == "f16") p.storage = SEMB_STORE_F16;
  else if (store == "bf16") p.storage = SEMB_STORE_BF16;
  else if (store == "f32") p.storage = SEMB_STORE_F32;
  else die_help();
  if (method == SEMB_CRS) {
    try {
      p.ngen = std::stoi(get("-ngen", false, "0"));
    } catch (const std::exception& e) {
      FAIL(std::string("bad numeric argument: ") + e.what());
    }
    const std::string dm = get("-dm", false, "abs");
    if (dm == "abs") p.dm_mode = SEMB_DM_ABS;
    else if (dm == "signed") p.dm_mode = SEMB_DM_SIGNED;
    else die_help();
  }

  const bool attrs = std::atoi(get("-attrs", false, "0").c_str()) != 0;
  p.attrs = attrs && p.mode == SEMB_BATCHED ? 1 : 0;

  semb_survey* survey = nullptr;
  check(semb_survey_load(path.c_str(), method, p.aph, &survey), "reading input");
  semb_gather_view v;
  check(semb_survey_view(survey, &v), "linearizing");
  if (v.ncdps == 0) FAIL("no traces within the offset aperture");

  semb_plan* plan = nullptr;
  check(semb_plan_create(&p, device, &plan), "creating the search");
  const auto beg = std::chrono::high_resolution_clock::now();
  check(semb_plan_upload(plan, &v), "uploading the gather");
  check(semb_plan_run(plan), "searching");
  const size_t n = (size_t)v.ncdps * v.ns;
  std::vector<int32_t> ctr(n);
  std::vector<float> str(n), stk(n);
  check(semb_plan_download(plan, ctr.data(), str.data(), stk.data()), "downloading results");
  const auto end = std::chrono::high_resolution_clock::now();
  semb_stats s;
  semb_plan_stats(plan, &s);
  const double t = std::chrono::duration<double>(end - beg).count();
  // the reference's rate: traces x samples x candidates / s, in 1e9 units
  // (CMP/OpenMP/src/main.cpp:240, CRS/OpenMP/src/main.cpp:327)
  const double rate = (double)s.trace_evals / 1e9 / t;
  char line[256];
  std::snprintf(line, sizeof(line), "Execution Time: %f, %s: %f", t,
                method == SEMB_CMP ? "Semblances-Trace/s" : "Mega-Semblances-Trace/s", rate);
  info(__FILE__, __LINE__, line);
  std::snprintf(line, sizeof(line), "Kernel Time: %f, Semblance evaluations/s: %.6e", s.ms_total * 1e-3,
                (double)s.evals / (s.ms_total * 1e-3));
  info(__FILE__, __LINE__, line);
  if (p.ngen > 0) {
    std::vector<float> av(n), bv(n), cv(n);
    check(semb_plan_download_abc(plan, av.data(), bv.data(), cv.data()), "downloading results");
    check(semb_survey_write_abc(survey, av.data(), bv.data(), cv.data(), str.data(), stk.data(), "."),
          "writing outputs");
  } else {
    check(semb_survey_write(survey, &p, ctr.data(), str.data(), stk.data(), "."), "writing outputs");
  }
  if (attrs) {
    // extra attribute files: aperture map (any form); second-best semblance and the
    // FP64 error of the pick (batched form)
    const std::string pre = method == SEMB_CMP ? "cmp." : "crs.";
    std::vector<int32_t> ap(v.ncdps);
    std::vector<float> buf(n);
    if (p.mode == SEMB_BATCHED) {
      std::vector<float> sem2(n), err(n);
      std::vector<int32_t> idx2(n);
      check(semb_plan_download_attrs(plan, sem2.data(), idx2.data(), err.data(), ap.data()), "downloading attributes");
      check(semb_survey_write_attr(survey, (pre + "coher2.su").c_str(), sem2.data(), "."), "writing outputs");
      check(semb_survey_write_attr(survey, (pre + "err64.su").c_str(), err.data(), "."), "writing outputs");
    } else {
      check(semb_plan_download_attrs(plan, nullptr, nullptr, nullptr, ap.data()), "downloading attributes");
    }
    for (int i = 0; i < v.ncdps; ++i)
      for (int q = 0; q < v.ns; ++q) buf[(size_t)i * v.ns + q] = (float)ap[i];
    check(semb_survey_write_attr(survey, (pre + "aperture.su").c_str(), buf.data(), "."), "writing outputs");
  }
  semb_plan_destroy(plan);
  semb_survey_free(survey);
  return EXIT_SUCCESS;
}
