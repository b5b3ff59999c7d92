// Written in the D programming language.

/**
   The time loop of DLBC with the timestep on the GPU.

   $(D runTimeloopGpu) replaces the body of $(D runTimeloop)
   (src/main.d:174-200): the lattice fields go to the device once
   ($(D lbgpu_upload)), the whole step (exchangeHalo, advectFields, the
   Shan-Chen force, collideFields) runs there, and the D fields are refreshed
   from the device ($(D lbgpu_download)) only when $(D dumpData) will write
   something, so that the reference's own output and checkpoint code
   (src/dlbc/io/io.d:198-213, src/dlbc/lb/io.d:56-101,
   src/dlbc/io/checkpoint.d:116-121) runs unchanged on the host fields.

   Hooks (src/dlbc/hooks.d:57-118): the reference registers its own
   stale-marking functions on postAdvectionHooks (src/dlbc/lb/density.d:338,
   src/dlbc/lb/force.d:131), which are harmless on refreshed fields.  Plugins
   whose hooks read or change the populations set $(D gpu.hostHooks = true):
   each step is then split at the hook points (lbgpu_advect, lbgpu_collide)
   and the fields are downloaded before and uploaded after every hook list.
   Plugins whose hooks sit only before advection and after collision also
   set $(D gpu.hooksAroundStep = true): each step is then one
   $(D lbgpu_step_host) call on the D fields, which stay the state.

   Errors: a nonzero status from the library is fatal, through writeLogF
   (src/dlbc/logging.d:255), as every fatal error of the reference is.

   Usage: add this module (src/dlbc/gpu/gpu.d) and dlbc.gpu.lbgpu
   (src/dlbc/gpu/lbgpu.d); its @("param") variables are read from a [gpu]
   section (enableGpu, precision, device, hostHooks, hooksAroundStep) once
   the module is in the parameter parser's module list (src/dlbc/parameters.d:366-370); link
   liblbgpu.so, and in main (src/main.d:153) call
   ---
   if ( enableGpu ) L.runTimeloopGpu(); else L.runTimeloop();
   ---

   This file is not compiled in this repository (there is no D toolchain
   here); the library calls it makes are the ones the Python driver
   (dlbc_gb300/driver.py) makes and the tests check.
*/
module dlbc.gpu.gpu;

import std.conv : to;
import std.string : fromStringz;

import dlbc.gpu.lbgpu;
import dlbc.io.checkpoint : cpFreq;
import dlbc.io.io : dumpData, dumpNow, enableIO, startOutput;
import dlbc.lattice;
import dlbc.lb.advection : postAdvectionHooks, preAdvectionHooks;
import dlbc.lb.collision : postCollisionHooks, preCollisionHooks;
import dlbc.lb.eqdist : eqDistForm;
import dlbc.lb.force : enableShanChen, gcc, globalAcc, gwc, psiForm;
import dlbc.lb.io : colourFreq, densityFreq, forceFreq, maskFreq, populationFreq, velocityFreq;
import dlbc.lb.lb : components, tau, timestep, timesteps;
import dlbc.logging;

/// Run the timestep on the GPU.
@("param") bool enableGpu;
/// Arithmetic form: "fp64" (the reference's numbers), "fp32", "fp16" or
/// "i16" (16-bit fixed-point storage; D3Q19, even z extent, BDist2).
@("param") string precision = "fp64";
/// CUDA device ordinal.
@("param") int device;
/// Refresh the fields around every hook list each step.
@("param") bool hostHooks;
/**
   With hostHooks: the plugins' hooks sit only on preAdvectionHooks and
   postCollisionHooks.  Each step is then one lbgpu_step_host call (input
   copies, kernels and output copies overlapped) between the two lists.  The
   reference's own postAdvectionHooks (markDensitiesAsStale, markPsiAsStale,
   src/dlbc/lb/density.d:338, src/dlbc/lb/force.d:131) run after the step,
   where they mark the host's cached fields stale as before.
*/
@("param") bool hooksAroundStep;

private lbgpu_handle* handle;

private void check(int rc, string what) {
  if ( rc != LBGPU_OK ) {
    writeLogF("lbgpu_%s failed (status %d): %s", what, rc, to!string(fromStringz(lbgpu_last_error(handle))));
  }
}

/**
   The C configuration from the reference's parameters.
*/
lbgpu_config makeConfig(T)(ref T L) if ( isLattice!T ) {
  lbgpu_config c;
  c.d = T.lbconn.d;
  c.q = T.lbconn.q;
  foreach(immutable i; 0..T.lbconn.d) c.gn[i] = to!int(L.gn[i]);
  c.components = components;
  c.shan_chen = enableShanChen ? 1 : 0;
  c.psi_form = cast(int) psiForm;
  c.eq_form = cast(int) eqDistForm;
  switch(precision) {
  case "fp64": c.precision = LBGPU_FP64; break;
  case "fp32": c.precision = LBGPU_FP32; break;
  case "fp16": c.precision = LBGPU_FP16; break;
  case "i16": c.precision = LBGPU_I16; break;
  default: writeLogF("gpu.precision must be fp64, fp32, fp16 or i16, not `%s'.", precision);
  }
  c.device = device;
  foreach(immutable f; 0..components) {
    c.tau[f] = tau[f];
    if ( gwc.length > 0 ) c.gwc[f] = gwc[f];
    if ( enableShanChen ) {
      foreach(immutable f2; 0..components) c.gcc[f][f2] = gcc[f][f2];
    }
  }
  foreach(immutable i; 0..T.lbconn.d) if ( globalAcc.length > 0 ) c.global_acc[i] = globalAcc[i];
  return c;
}

private void upload(T)(ref T L) {
  const(double)*[LBGPU_MAX_COMPONENTS] f;
  foreach(immutable i, ref e; L.fluids) f[i] = cast(const(double)*) e.arr._data.ptr;
  check(lbgpu_upload(handle, f.ptr, cast(const(int)*) L.mask.arr._data.ptr), "upload");
}

/// One timestep from the D fields to the D fields (lbgpu_step_host).
private void stepHost(T)(ref T L) {
  const(double)*[LBGPU_MAX_COMPONENTS] fin;
  double*[LBGPU_MAX_COMPONENTS] fout;
  foreach(immutable i, ref e; L.fluids) {
    fin[i] = cast(const(double)*) e.arr._data.ptr;
    fout[i] = cast(double*) e.arr._data.ptr;
  }
  check(lbgpu_step_host(handle, fin.ptr, cast(const(int)*) L.mask.arr._data.ptr, fout.ptr), "step_host");
}

private void download(T)(ref T L) {
  double*[LBGPU_MAX_COMPONENTS] f;
  foreach(immutable i, ref e; L.fluids) f[i] = cast(double*) e.arr._data.ptr;
  check(lbgpu_download(handle, f.ptr), "download");
}

/**
   Copy the last step's force (physical sites, [x][y][z][d]) into the haloed
   force fields that dumpLBData writes.
*/
private void downloadForce(T)(ref T L) {
  import std.algorithm : reduce;
  immutable size_t n = reduce!"a * b"(cast(size_t) 1, L.lengths[]);
  enum d = T.lbconn.d;
  double[][LBGPU_MAX_COMPONENTS] buf;
  double*[LBGPU_MAX_COMPONENTS] ptrs;
  foreach(immutable i; 0..components) {
    buf[i].length = n * d;
    ptrs[i] = buf[i].ptr;
  }
  check(lbgpu_force(handle, ptrs.ptr), "force");
  foreach(immutable i, ref e; L.force) {
    size_t k = 0;
    foreach(immutable p, ref v; e) {  // physical sites in row-major order
      foreach(immutable vd; 0..d) v[vd] = buf[i][k * d + vd];
      ++k;
    }
  }
}

/**
   Whether dumpData (src/dlbc/io/io.d:198-213) writes anything at t.
*/
private bool dumpsAt(int t) {
  if ( ! enableIO || t < startOutput ) return false;
  return dumpNow(cpFreq, t) || dumpNow(populationFreq, t) || dumpNow(densityFreq, t) || dumpNow(colourFreq, t)
    || dumpNow(velocityFreq, t) || dumpNow(forceFreq, t) || dumpNow(maskFreq, t);
}

/**
   The time loop on the GPU.  Equivalent to runTimeloop (src/main.d:174-200)
   on one process; with gpu.precision = fp64 the fields it dumps are bit for
   bit the reference's.
*/
void runTimeloopGpu(T)(ref T L) if ( isLattice!T ) {
  if ( L.lengths != L.gn ) {
    writeLogF("The GPU timestep runs the whole lattice in one process: start DLBC on one MPI rank.");
  }
  auto cfg = makeConfig(L);
  check(lbgpu_create(&cfg, &handle), "create");
  scope(exit) {
    lbgpu_destroy(handle);
    handle = null;
  }
  upload(L);
  if ( forceFreq > 0 ) check(lbgpu_set_record_force(handle, 1), "set_record_force");
  writeLogRN("Running the timestep on GPU %d (%s).", device, precision);

  while ( timestep < timesteps ) {
    if ( hostHooks && hooksAroundStep ) {
      // the D fields hold the state between steps: they go through the
      // timestep in one call and come back for the post-collision hooks
      ++timestep;
      writeLogRN("Starting timestep %d", timestep);
      preAdvectionHooks.execute(L);
      stepHost(L);
      postAdvectionHooks.execute(L);
      postCollisionHooks.execute(L);
    }
    else if ( hostHooks ) {
      ++timestep;
      writeLogRN("Starting timestep %d", timestep);
      download(L);
      preAdvectionHooks.execute(L);
      upload(L);
      check(lbgpu_advect(handle), "advect");
      download(L);
      postAdvectionHooks.execute(L);
      preCollisionHooks.execute(L);
      upload(L);
      check(lbgpu_collide(handle), "collide");
      download(L);
      postCollisionHooks.execute(L);
      upload(L);
    }
    else {
      // all steps up to the next one that writes output, in one call
      int k = 1;
      while ( timestep + k < timesteps && ! dumpsAt(timestep + k) ) ++k;
      check(lbgpu_step(handle, k), "step");
      timestep += k;
      writeLogRN("Completed timestep %d", timestep);
      if ( dumpsAt(timestep) ) download(L);
    }
    if ( dumpsAt(timestep) && dumpNow(forceFreq, timestep) ) downloadForce(L);
    L.dumpData(timestep);
  }
  check(lbgpu_synchronize(handle), "synchronize");
}
