#!/usr/bin/env bash
# Compile the reference's own sources (unmodified, read in place from /root/reference) against the
# project's serial SYCL host shim (oracle/ref/shim) and the driver oracle/ref/ref_driver.cpp, one
# binary per scheme flavour, into oracle/_ref/<flavour>/xfluids_ref. The reference's build system
# is not used; the macros below are the ones its cmake/init_options.cmake and init_sample.cmake
# would set for these flavours. Used only to pin the oracle (test infrastructure).
#
# usage: bash oracle/ref/build_ref.sh [flavour ...]   (default: all flavours)
#        bash oracle/ref/build_ref.sh --root           (print the reference location and exit)
# The reference location is $XF_REFERENCE, by default the read-only checkout of this container.
set -euo pipefail
REF=${XF_REFERENCE:-/root/reference}
if [ "${1:-}" = "--root" ]; then echo "$REF"; exit 0; fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$(cd "$HERE/.." && pwd)/_ref
[ -d "$REF/src" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
ln -sfn "$REF/runtime.dat" "$OUT/runtime.dat"   # WorkDir search (external/fworkdir.hpp:12-26)

# flavour: name | macros | ini sample dir | mixture dir (relative to the work dir)
FLAVOURS=(
  "ncop_w5_llf|-DSCHEME_ORDER=5 -DArtificial_type=2 -DNUM_SPECIES=1 -DNUM_COP=0 -DNCOP_Gamma=1.4 -DThermo=1|2D-EulerVortex|runtime.dat/NO-COP"
  "ncop_w7_llf|-DSCHEME_ORDER=7 -DArtificial_type=2 -DNUM_SPECIES=1 -DNUM_COP=0 -DNCOP_Gamma=1.4 -DThermo=1|2D-EulerVortex|runtime.dat/NO-COP"
  "ncop_w5_roe|-DSCHEME_ORDER=5 -DArtificial_type=1 -DNUM_SPECIES=1 -DNUM_COP=0 -DNCOP_Gamma=1.4 -DThermo=1|2D-EulerVortex|runtime.dat/NO-COP"
  "ncop_w5_glf|-DSCHEME_ORDER=5 -DArtificial_type=3 -DNUM_SPECIES=1 -DNUM_COP=0 -DNCOP_Gamma=1.4 -DThermo=1|2D-EulerVortex|runtime.dat/NO-COP"
  "cop4g_w5_llf_nasa|-DCOP -DSCHEME_ORDER=5 -DArtificial_type=2 -DThermo=1|1D-X-Y-Z/insert-st|runtime.dat/1d-mc-insert-shock-tube"
  "cop5_w7_llf_janaf|-DCOP -DSCHEME_ORDER=7 -DArtificial_type=2 -DThermo=0|1D-X-Y-Z/insert-st|cases/mixing5"
  # WENO-CU6 (SCHEME_ORDER=6, schemes_device.hpp:18-19)
  "ncop_w6_llf|-DSCHEME_ORDER=6 -DArtificial_type=2 -DNUM_SPECIES=1 -DNUM_COP=0 -DNCOP_Gamma=1.4 -DThermo=1|2D-EulerVortex|runtime.dat/NO-COP"
  "cop5_w6_roe_janaf|-DCOP -DSCHEME_ORDER=6 -DArtificial_type=1 -DThermo=0|1D-X-Y-Z/insert-st|cases/mixing5"
  # viscous, heat-conduction and diffusion fluxes (init_options.cmake:81-91)
  "cop5_w5_llf_janaf_visc|-DCOP -DSCHEME_ORDER=5 -DArtificial_type=2 -DThermo=0 -UVisc -DVisc=1 -DVisc_Heat=1 -DVisc_Diffu=1|1D-X-Y-Z/insert-st|cases/mixing5"
  # PositivityPreserving on (init_sample.cmake:218-219 sets POSP=1 for the samples that use it)
  "ncop_w5_llf_pp|-DSCHEME_ORDER=5 -DArtificial_type=2 -DNUM_SPECIES=1 -DNUM_COP=0 -DNCOP_Gamma=1.4 -DThermo=1 -UPOSP -DPOSP=1|2D-EulerVortex|runtime.dat/NO-COP"
  "cop5_w5_llf_janaf_pp|-DCOP -DSCHEME_ORDER=5 -DArtificial_type=2 -DThermo=0 -UPOSP -DPOSP=1|1D-X-Y-Z/insert-st|cases/mixing5"
)

SRCS=(
  src/Fluids.cpp src/XFLUIDS.cpp src/solver_Ini/Ini_block.cpp src/solver_BCs/BCs_block.cpp
  src/solver_UpdateStates/UpdateStates_block.cpp src/read_ini/src/constructor.cpp src/read_ini/src/gpucopy.cpp
  src/read_ini/src/iniset.cpp src/read_ini/src/print.cpp src/read_ini/src/reaction.cpp src/read_ini/src/thermal.cpp
  src/read_ini/src/viscfit.cpp src/read_ini/settings/read_json.cpp src/read_ini/inishape/inishape.cpp
  src/read_ini/outformat/outformat.cpp src/read_grid/readgrid.cpp external/timer/timer.cpp
  external/strsplit/strsplit.cpp external/ndassign/ndassign.cpp external/kattribute/attribute.cpp
)

# the mixture of the 5-species mixing layer is not among the reference's runtime.dat cases:
# species list and case header supplied here (runtime.dat itself is used unchanged)
mkdir -p "$OUT/cases/mixing5"
printf 'H2 O2 N2 H2O AR\n1 1 1 1 1\n1 1 1 1 1\n' > "$OUT/cases/mixing5/species_list.dat"
printf '#pragma once\n#define NUM_SPECIES 5\n' > "$OUT/cases/mixing5/case_setup.h"

want=("$@")
for fl in "${FLAVOURS[@]}"; do
  IFS='|' read -r name macros sample mixture <<< "$fl"
  if [ ${#want[@]} -gt 0 ] && [[ ! " ${want[*]} " =~ " $name " ]]; then continue; fi
  dir="$OUT/$name"
  mkdir -p "$dir/obj"
  if [ -x "$dir/xfluids_ref" ] && [ "$dir/xfluids_ref" -nt "$HERE/ref_driver.cpp" ] && [ "$dir/xfluids_ref" -nt "$HERE/shim/sycl/sycl.hpp" ]; then
    continue
  fi
  if [[ "$mixture" == runtime.dat/* ]]; then mixinc="$REF/$mixture"; else mixinc="$OUT/$mixture"; fi
  flags=(-std=c++17 -O2 -U_FORTIFY_SOURCE -ffp-contract=off -w -include cstdint -include memory -include cstring
         -D__ACPP__ -DUSE_DOUBLE -DEIGEN_ALLOC=0 -DESTIM_NAN=1 -DESTIM_OUT=0 -D__SYNC_TIMER_=1 -DPOSP=0
         -DCOP_CHEME=0 -DNUM_REA=1 -DVisc=0 $macros
         "-DINI_SAMPLE=\"ini-$name\"" "-DRFile=\"/$mixture\"" "-DIniFile=\"$dir/case.json\"" "-DRPath=\"/runtime.dat\""
         -I"$HERE/shim" -I"$REF/src" -I"$REF/src/include" -I"$REF/external" -I"$mixinc"
         -I"$REF/src/solver_Ini/sample/$sample" -I"$REF/src/solver_Reconstruction/viscosity/Fourth_Order"
         -I"$REF/src/solver_Reconstruction/FDM_Method" -I"$REF/src/solver_Reconstruction/FDM_Method/positive-definite_eigen"
         -I"$REF/src/solver_Reconstruction")
  pids=()
  for s in "${SRCS[@]}" "DRIVER"; do
    if [ "$s" = DRIVER ]; then src="$HERE/ref_driver.cpp"; obj="$dir/obj/ref_driver.o"
    else src="$REF/$s"; obj="$dir/obj/$(echo "$s" | tr '/' '_').o"; fi
    g++ "${flags[@]}" -c "$src" -o "$obj" &
    pids+=($!)
    if [ ${#pids[@]} -ge "$(nproc)" ]; then wait "${pids[0]}"; pids=("${pids[@]:1}"); fi
  done
  for p in "${pids[@]}"; do wait "$p"; done
  g++ -o "$dir/xfluids_ref" "$dir"/obj/*.o
  echo "built $dir/xfluids_ref"
done

# The reference's own XFLUIDS executable (its main.cpp and every source but src/Fluids.cpp) linked
# with the drop-in class Fluid of xfluids_gb300/host/Fluids_gb300.cpp over libxfluids_gb300.so:
# shows that the boundary compiles and links against the unmodified reference headers.
LIBDIR=$(cd "$HERE/../.." && pwd)/xfluids_gb300/_build
if [ -f "$LIBDIR/libxfluids_gb300.so" ] && { [ ${#want[@]} -eq 0 ] || [[ " ${want[*]} " =~ " dropin " ]]; }; then
  # a single gas and the viscous 5-species mixture (Visc, Visc_Heat, Visc_Diffu: xfg_set_transport)
  for fl in "${FLAVOURS[@]}"; do
    IFS='|' read -r name macros sample mixture <<< "$fl"
    case "$name" in ncop_w5_llf|cop5_w5_llf_janaf_visc) ;; *) continue ;; esac
    base="$OUT/$name"
    d="$OUT/dropin_$name"
    [ -d "$base/obj" ] || continue
    mkdir -p "$d"
    if [[ "$mixture" == runtime.dat/* ]]; then mixinc="$REF/$mixture"; else mixinc="$OUT/$mixture"; fi
    dflags=(-std=c++17 -O2 -U_FORTIFY_SOURCE -ffp-contract=off -w -include cstdint -include memory -include cstring
            -D__ACPP__ -DUSE_DOUBLE -DEIGEN_ALLOC=0 -DESTIM_NAN=1 -DESTIM_OUT=0 -D__SYNC_TIMER_=1 -DPOSP=0
            -DCOP_CHEME=0 -DNUM_REA=1 -DVisc=0 $macros
            "-DINI_SAMPLE=\"ini-dropin\"" "-DRFile=\"/$mixture\"" "-DIniFile=\"$d/case.json\"" "-DRPath=\"/runtime.dat\""
            -I"$HERE/shim" -I"$REF/src" -I"$REF/src/include" -I"$REF/external" -I"$mixinc"
            -I"$REF/src/solver_Ini/sample/$sample" -I"$REF/src/solver_Reconstruction/viscosity/Fourth_Order"
            -I"$REF/src/solver_Reconstruction/FDM_Method" -I"$REF/src/solver_Reconstruction/FDM_Method/positive-definite_eigen"
            -I"$REF/src/solver_Reconstruction" -I"$HERE/../../include")
    g++ "${dflags[@]}" -c "$HERE/../../xfluids_gb300/host/Fluids_gb300.cpp" -o "$d/Fluids_gb300.o"
    g++ "${dflags[@]}" -c "$REF/src/main.cpp" -o "$d/main.o"
    objs=()
    for o in "$base"/obj/*.o; do
      case "$(basename "$o")" in src_Fluids.cpp.o|ref_driver.o) ;; *) objs+=("$o") ;; esac
    done
    g++ -o "$d/xfluids_gb300_dropin" "$d/Fluids_gb300.o" "$d/main.o" "${objs[@]}" -L"$LIBDIR" -lxfluids_gb300 -Wl,-rpath,"$LIBDIR"
    echo "built $d/xfluids_gb300_dropin"
  done
fi
