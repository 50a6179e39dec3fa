#include "System.hpp"

#include <cmath>
#include <initializer_list>
#include <utility>
#include <fstream>
#include <iostream>
#include <sstream>

#include "../../include/cflbm.h"

System::System() { read("input.in"); }
System::System(const std::string &path) { read(path); }

void System::read(const std::string &path) {
  cs2 = 1.0 / 3.0;
  cs = std::sqrt(cs2);
  std::ifstream input(path);
  input >> rho0 >> R >> Re;
  input >> u0 >> Time >> inter;
  input >> sx >> sy >> sz;
  ok = static_cast<bool>(input);
  Ma = u0 / cs;
  miu = rho0 * u0 * R / Re;
  tau = u0 * R / Re / cs2;
  // The reference recomputes the run length from R and miu.
  Time = std::pow(2 * R, 2) / miu;
  inter = Time / 10;

  // Extension keys.  A value that names nothing known is an error (ok = false,
  // `error` names the key): a misspelt profile or storage must not fall back
  // to another solver silently.
  auto pick = [&](const std::string &key, const std::string &v,
                  std::initializer_list<std::pair<const char *, int>> names, int &dst) {
    for (const auto &nv : names)
      if (v == nv.first) {
        dst = nv.second;
        return;
      }
    std::string want;
    for (const auto &nv : names) want += (want.empty() ? "" : ", ") + std::string(nv.first);
    if (error.empty())
      error = "input.in: cflbm." + key + " has unknown value '" + v + "' (expected one of " +
              want + ")";
  };
  std::string line;
  while (std::getline(input, line)) {
    std::istringstream ls(line);
    std::string key;
    ls >> key;
    if (key.rfind("cflbm.", 0) != 0) continue;
    key = key.substr(6);
    ext_keys.push_back(key);
    std::string v;
    if (key == "lattice") ls >> lattice;
    else if (key == "steps") ls >> Time;
    else if (key == "inter") ls >> inter;
    else if (key == "center") ls >> cx >> cy >> cz;
    else if (key == "diam") ls >> diam;
    else if (key == "perturb") ls >> perturb;
    else if (key == "seed") ls >> seed;
    else if (!(ls >> v)) {
      if (error.empty()) error = "input.in: cflbm." + key + " has no value";
    } else if (key == "profile")
      pick(key, v, {{"channel", CFLBM_PROFILE_CHANNEL}, {"ref2d", CFLBM_PROFILE_REF2D},
                    {"ref3d", CFLBM_PROFILE_REF3D}, {"ref2ds", CFLBM_PROFILE_REF2DS}},
           profile);
    else if (key == "storage")
      pick(key, v, {{"fp64", CFLBM_STORE_FP64}, {"fp32", CFLBM_STORE_FP32},
                    {"fp16dev", CFLBM_STORE_FP16DEV}}, storage);
    else if (key == "compute")
      pick(key, v, {{"fp64", CFLBM_COMPUTE_FP64}, {"fp32", CFLBM_COMPUTE_FP32},
                    {"df64", CFLBM_COMPUTE_DF64}}, compute);
    else if (key == "rounding")
      pick(key, v, {{"stochastic", CFLBM_ROUND_STOCHASTIC}, {"nearest", CFLBM_ROUND_NEAREST}},
           rounding);
    else if (key == "geom")
      pick(key, v, {{"none", CFLBM_GEOM_NONE}, {"cylinder", CFLBM_GEOM_CYLINDER},
                    {"sphere", CFLBM_GEOM_SPHERE}}, geom);
    else if (key == "wall_y" || key == "wall_z")
      pick(key, v, {{"freeslip", CFLBM_WALL_FREESLIP}, {"noslip", CFLBM_WALL_NOSLIP},
                    {"periodic", CFLBM_WALL_PERIODIC}}, key == "wall_y" ? wall_y : wall_z);
    else if (error.empty())
      error = "input.in: unknown key cflbm." + key;
  }
  if (lattice != CFLBM_D2Q9 && lattice != CFLBM_D3Q27 && error.empty())
    error = "input.in: cflbm.lattice must be 9 or 27";
  ext_error = !error.empty();
  if (!error.empty()) ok = false;
  else if (!ok) error = "could not read the nine numbers of " + path;
  if (inter <= 0) inter = 1;
}

void System::Monitor() {
  // Same text as the reference's System::Monitor ("3D.../System.cpp:25-41").
  std::cout << "============================" << std::endl
            << "3D Cylinder Flow" << std::endl
            << "Re    =" << Re << std::endl
            << "Ma    =" << Ma << std::endl
            << "rho   =" << rho0 << std::endl
            << "miu   =" << miu << std::endl
            << "tau   =" << tau << std::endl
            << "Time  =" << Time << std::endl
            << "inter =" << inter << std::endl
            << "nx    =" << sx << std::endl
            << "ny    =" << sy << std::endl
            << "nz    =" << sz << std::endl
            << "============================" << std::endl;
}
