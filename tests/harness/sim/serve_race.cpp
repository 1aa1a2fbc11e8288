// The serving layer's host threading under ThreadSanitizer, on the host
// simulation of the device side: a server with 4 worker threads solves
// sixteen small CCSD(T) requests submitted back to back (the last six of one
// shape, which the slots take in lockstep batches) while another thread polls
// its statistics.  Prints one line per result; ThreadSanitizer reports any
// data race on stderr.
#include <algorithm>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>
#include "gbcc.h"

struct Sys { int No, Nv, NG; std::vector<double> eh, ep, g; };

Sys make(int No, int Nv, int NG, unsigned seed) {
  std::mt19937_64 r(seed);
  std::normal_distribution<double> n(0.0, 0.03);
  std::uniform_real_distribution<double> uh(-1.5, -0.5), up(0.2, 3.0);
  Sys s{No, Nv, NG, {}, {}, {}};
  int Np = No + Nv;
  s.g.assign((size_t)NG * Np * Np, 0.0);
  for (int G = 0; G < NG; ++G)
    for (int p = 0; p < Np; ++p)
      for (int q = p; q < Np; ++q) {
        double v = n(r);
        s.g[G + NG * (p + Np * q)] = v;
        s.g[G + NG * (q + Np * p)] = v;
      }
  for (int i = 0; i < No; ++i) s.eh.push_back(uh(r));
  for (int a = 0; a < Nv; ++a) s.ep.push_back(up(r));
  std::sort(s.eh.begin(), s.eh.end());
  std::sort(s.ep.begin(), s.ep.end());
  return s;
}

int main() {
  gbcc_server_opts so;
  gbcc_server_opts_default(&so);
  so.slots = 4;
  gbcc_server *srv = nullptr;
  if (gbcc_server_create(&so, &srv) != GBCC_OK) { std::puts("create failed"); return 1; }
  std::vector<Sys> sys;
  for (int k = 0; k < 10; ++k) sys.push_back(make(2 + k % 2, 4 + k % 3, 8, 100 + k));
  for (int k = 0; k < 6; ++k) sys.push_back(make(2, 5, 8, 200 + k));
  std::vector<int64_t> ids(sys.size());
  std::thread poller([&]() {
    for (int t = 0; t < 200; ++t) {
      int p, r; int64_t b;
      gbcc_server_stats(srv, &p, &r, &b);
      std::this_thread::yield();
    }
  });
  for (size_t k = 0; k < sys.size(); ++k) {
    gbcc_ccsd_in in{};
    in.No = sys[k].No; in.Nv = sys[k].Nv; in.NG = sys[k].NG;
    in.eps_h = sys[k].eh.data(); in.eps_p = sys[k].ep.data(); in.gamma = sys[k].g.data();
    gbcc_ccsd_opts o;
    gbcc_ccsd_opts_default(&o);
    o.mixer = 1; o.max_residua = 5; o.max_iterations = 30;
    o.energy_convergence = 1e-10; o.amplitudes_convergence = 1e-8;
    if (gbcc_server_submit(srv, &in, &o, 1, &ids[k]) != GBCC_OK) { std::puts("submit failed"); return 1; }
  }
  for (size_t k = 0; k < sys.size(); ++k) {
    gbcc_result res;
    int st = gbcc_server_wait(srv, ids[k], &res);
    std::printf("id %lld st %d status %d E %.12f Et %.3e it %d\n", (long long)ids[k], st,
                res.status, res.e_ccsd, res.e_t, res.iterations);
  }
  poller.join();
  gbcc_server_destroy(srv);
  return 0;
}
