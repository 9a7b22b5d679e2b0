// Control block of the device-resident time loop, shared by host and device.
#pragma once

namespace weno {

struct StepCtl {
  double dt;                     // step size of the current step
  double t;                      // simulated time after the completed steps
  double t_final;                // < 0: step-count mode
  double cfl_dx;                 // CFL * dx
  unsigned long long cmax_bits;  // running max of c + |u| (non-negative doubles order as integers)
  int cmax_preset;               // 1: cmax_bits already holds this step's maximum (first step of a run
                                 //    loaded from the driver's array, whose primitive channels set dt)
  int active;                    // 0 once the loop condition fails: the step's kernels return at once
  long long steps;               // completed steps
  long long max_steps;           // cap on completed steps
  int status;                    // 0 ok; 1 non-finite wave speed seen
};

}  // namespace weno
