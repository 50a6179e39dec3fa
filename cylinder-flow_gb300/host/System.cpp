#include "System.hpp"

#include <cmath>
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

  std::string line;
  while (std::getline(input, line)) {
    std::istringstream ls(line);
    std::string key;
    ls >> key;
    if (key.rfind("cflbm.", 0) != 0) continue;
    key = key.substr(6);
    std::string v;
    if (key == "lattice") ls >> lattice;
    else if (key == "steps") ls >> Time;
    else if (key == "inter") ls >> inter;
    else if (key == "center") ls >> cx >> cy >> cz;
    else if (key == "diam") ls >> diam;
    else if (key == "perturb") ls >> perturb;
    else if (key == "seed") ls >> seed;
    else if (ls >> v) {
      if (key == "profile")
        profile = v == "channel" ? CFLBM_PROFILE_CHANNEL
                  : v == "ref2d" ? CFLBM_PROFILE_REF2D : CFLBM_PROFILE_REF3D;
      else if (key == "storage")
        storage = v == "fp32" ? CFLBM_STORE_FP32 : v == "fp16dev" ? CFLBM_STORE_FP16DEV
                                                                   : CFLBM_STORE_FP64;
      else if (key == "compute")
        compute = v == "fp32" ? CFLBM_COMPUTE_FP32 : v == "df64" ? CFLBM_COMPUTE_DF64
                                                                 : CFLBM_COMPUTE_FP64;
      else if (key == "geom")
        geom = v == "cylinder" ? CFLBM_GEOM_CYLINDER : v == "sphere" ? CFLBM_GEOM_SPHERE
                                                                      : CFLBM_GEOM_NONE;
      else if (key == "wall_y" || key == "wall_z") {
        int w = v == "noslip" ? CFLBM_WALL_NOSLIP : v == "periodic" ? CFLBM_WALL_PERIODIC
                                                                    : CFLBM_WALL_FREESLIP;
        (key == "wall_y" ? wall_y : wall_z) = w;
      }
    }
  }
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
