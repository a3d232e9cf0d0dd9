#!/usr/bin/env bash
# Regenerates the mechanism and gas-model fixtures under tests/golden/mech/.
#
# It builds the reference's own vendored Lua 5.4.3 + lpeg (extern/lua-5.4.3) in a
# scratch directory, assembles the species database exactly as
# src/gas/species-database/makefile does, and runs the reference's pre-processors
# prep_gas.lua and prep_chem.lua on the mechanism inputs.  The machine-readable
# files it writes are what the reference's D code reads at run time
# (src/kinetics/chemistry_update.d:42-137, src/gas/composite_gas.d:37-120).
# The reference's own sample data used by its unit tests is copied verbatim.
#
# Usage: tests/golden/make_fixtures.sh [REFERENCE_DIR]   (needs gcc and make)
set -euo pipefail
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/mech
WORK=$(mktemp -d /tmp/gdtk_fixtures.XXXXXX)
trap 'rm -rf "$WORK"' EXIT

cp -r "$REF/extern/lua-5.4.3" "$WORK/lua"
chmod -R u+w "$WORK/lua"
(cd "$WORK/lua" && make linux local > "$WORK/lua-build.log" 2>&1)
LUA=$WORK/lua/install/bin/dgd-lua

mkdir -p "$WORK/dgd/data" "$WORK/dgd/lib"
(cd "$REF/src/gas/species-database" && awk '$1 !~ "#" {print $1}' < species-list.txt | xargs cat defaults.lua) \
    > "$WORK/dgd/data/species-database.lua"
cp "$REF/src/gas/species-database/species-list.txt" "$WORK/dgd/data/"
cp "$REF/src/gas/species-database/collision-integrals/"*.lua "$WORK/dgd/data/"   # two-temperature gas files
cp "$REF/src/kinetics/reaction.lua" "$REF/src/kinetics/lex_elems.lua" "$REF/src/kinetics/mechanism.lua" "$WORK/dgd/lib/"
# The species check of reaction.lua (checkEquationSpecies) indexes every parsed participant, but the
# '(+ M)' marker of a pressure-dependent reaction parses to a plain string, so prep_chem stops with
# "Species nil ... not found".  In the scratch copy only, such entries are treated as the collider M.
sed -i 's/local sp = p\[2\]$/local sp = type(p) == "table" and p[2] or "M"/' "$WORK/dgd/lib/reaction.lua"
export DGD=$WORK/dgd
export DGD_LUA_PATH="$WORK/dgd/lib/?.lua;;"
export DGD_LUA_CPATH="$WORK/lua/install/lib/?.so;;"

mkdir -p "$OUT"
prep() {  # name gas-input mechanism-input
    (cd "$WORK" && "$LUA" "$REF/src/gas/prep_gas.lua" "$2" "$1-gas.lua" > "$WORK/$1-prep.log" 2>&1 \
        && "$LUA" "$REF/src/kinetics/prep_chem.lua" "$1-gas.lua" "$3" "$1-chem.lua" >> "$WORK/$1-prep.log" 2>&1) \
        || { cat "$WORK/$1-prep.log"; exit 1; }
    # Drop the time-stamp comment so that regenerated files compare equal.
    grep -v '^-- Auto-generated' "$WORK/$1-gas.lua" > "$OUT/$1-gas.lua"
    cp "$WORK/$1-chem.lua" "$OUT/$1-chem.lua"
}
KIN=$REF/examples/kinetics
prep park5  "$HERE/inputs/air5-park.inp"                              "$HERE/inputs/park5-arrhenius.lua"
prep j92    "$KIN/hydrogen-ignition-delay/Jachimowski-1992-species.inp" "$KIN/hydrogen-ignition-delay/Jachimowski-1992.lua"
prep n2     "$KIN/fixed-volume-reactor-n2/nitrogen-2sp.inp"            "$KIN/fixed-volume-reactor-n2/nitrogen-2sp-2r-Keq.lua"
prep gupta5 "$KIN/air-chemistry-1T/air-5sp-1T.inp"                     "$KIN/air-chemistry-1T/GuptaEtAl-air-reactions.lua"
# pressure-dependent (Troe) reactions: F_cent given (Stanford-2011), and a, T3, T1, T2 (DRM19 methane)
prep stanford "$KIN/hydrogen-ignition-delay/Stanford-2011-species.inp"  "$KIN/hydrogen-ignition-delay/Stanford-2011.lua"
prep drm19  "$KIN/methane-combustion-w-drm19/drm19-prep-gas.inp"       "$KIN/methane-combustion-w-drm19/drm19-prep-chem.inp"
# Two-temperature air (Park 1993, 5 species): gas, reactions (Park 2-T rates) and energy exchange
# (Landau-Teller with Millikan-White and Park's high-temperature correction; Marrone-Treanor coupling),
# the inputs of examples/lmr/3D/cylinder-larc, through prep_gas, prep_chem and prep_kinetics.
LARC=$REF/examples/lmr/3D/cylinder-larc
(cd "$WORK" && "$LUA" "$REF/src/gas/prep_gas.lua" "$LARC/gm-air-5sp-2T.inp" park2t-gas.lua > park2t-prep.log 2>&1 \
    && "$LUA" "$REF/src/kinetics/prep_chem.lua" park2t-gas.lua "$LARC/rm-park-5sp-2T.inp" park2t-chem.lua \
        >> park2t-prep.log 2>&1 \
    && "$LUA" "$REF/src/kinetics/prep_kinetics.lua" park2t-gas.lua park2t-chem.lua "$LARC/eem-park-5sp-2T.inp" \
        park2t-eem.lua >> park2t-prep.log 2>&1) || { cat "$WORK/park2t-prep.log"; exit 1; }
grep -v '^-- Auto-generated' "$WORK/park2t-gas.lua" > "$OUT/park2t-gas.lua"
cp "$WORK/park2t-chem.lua" "$WORK/park2t-eem.lua" "$OUT/"
# The Marrone-Treanor forms on the same air (rate_constant.d:395-560, exchange_chemistry_coupling.d:133-227;
# no reference example uses them): N2 dissociation as a Marrone-Treanor rate (T_D/U = 3) over its Arrhenius
# rate, coupled by MarroneTreanorDissociation; O2 dissociation as a Modified-Marrone-Treanor rate over its
# Park rate with a constant non-Boltzmann factor, coupled by ModifiedMarroneTreanorDissociation; NO
# dissociation unchanged.  The model parameters are test values; theta_v are the species' vibrational
# temperatures.
sed -e "s|fr={'Park', A=7.0e21, n=-1.60, C=113200.0, s=0.5},|fr={'Marrone-Treanor', D='N2', TD_on_U=3.0, theta_v=3393.44, rate={'Arrhenius', A=7.0e21, n=-1.60, C=113200.0}},|" \
    -e "s|fr={'Park', A=2.0e21, n=-1.5, C=59500.0, s=0.5},|fr={'Modified-Marrone-Treanor', D_sp='O2', Thetav=2273.54, aU=0.15, Ustar=40000.0, rate={'Park', A=2.0e21, n=-1.5, C=59500.0, s=0.5}, non_boltzmann_correction={model='constant', factor=0.9}},|" \
    "$LARC/rm-park-5sp-2T.inp" > "$WORK/rm-mt.inp"
grep -q "Modified-Marrone-Treanor" "$WORK/rm-mt.inp" && grep -q "'Marrone-Treanor'" "$WORK/rm-mt.inp"
sed '/^ChemistryCouplingMechanism{/,$d' "$LARC/eem-park-5sp-2T.inp" > "$WORK/eem-mt.inp"
cat >> "$WORK/eem-mt.inp" <<'EOF2'
ChemistryCouplingMechanism{
    reaction_labels = {"r1"},
    rate = "Marrone-Treanor",
    coupling_model = {model="MarroneTreanorDissociation", TD_on_U=3.0, Thetav=3393.44}
}
ChemistryCouplingMechanism{
    reaction_labels = {"r2"},
    rate = "Marrone-Treanor",
    coupling_model = {model="ModifiedMarroneTreanorDissociation", Thetav=2273.54, aU=0.15, Ustar=40000.0, non_boltzmann=0.1}
}
ChemistryCouplingMechanism{
    reaction_labels = {"r3"},
    rate = "Marrone-Treanor",
    coupling_model = {model="ImpartialDissociation"}
}
EOF2
(cd "$WORK" && "$LUA" "$REF/src/kinetics/prep_chem.lua" park2t-gas.lua rm-mt.inp park2tmt-chem.lua > park2tmt-prep.log 2>&1 \
    && "$LUA" "$REF/src/kinetics/prep_kinetics.lua" park2t-gas.lua park2tmt-chem.lua eem-mt.inp park2tmt-eem.lua \
        >> park2tmt-prep.log 2>&1) || { cat "$WORK/park2tmt-prep.log"; exit 1; }
cp "$WORK/park2tmt-chem.lua" "$WORK/park2tmt-eem.lua" "$OUT/"
# A large mechanism: the 75-species, 474-reaction C2H2/C2H4 model of examples/kinetics/acetylene-ignition-
# delay (Chemkin format), converted by the reference's chemkin2eilmer (which runs prep-gas itself) and
# prep_chem, as that example's prep-ignition.sh does.
mkdir -p "$WORK/bin"
printf '#!/bin/sh\nexec "%s" "%s" "$@"\n' "$LUA" "$REF/src/gas/prep_gas.lua" > "$WORK/bin/prep-gas"
chmod +x "$WORK/bin/prep-gas"
(cd "$WORK" && PATH="$WORK/bin:$PATH" "$LUA" "$REF/src/kinetics/chemkin2eilmer.lua" \
        "$KIN/acetylene-ignition-delay/mech.txt" c2h2-gas.lua c2h2-reac.lua > c2h2-prep.log 2>&1 \
    && "$LUA" "$REF/src/kinetics/prep_chem.lua" c2h2-gas.lua c2h2-reac.lua c2h2-chem.lua >> c2h2-prep.log 2>&1) \
    || { cat "$WORK/c2h2-prep.log"; exit 1; }
grep -v '^-- Auto-generated' "$WORK/c2h2-gas.lua" > "$OUT/c2h2-gas.lua"
cp "$WORK/c2h2-chem.lua" "$OUT/c2h2-chem.lua"
# Arrhenius2, Lindemann-Hinshelwood and Yungster-Rabinowitz forms (no reference example uses them)
prep h2o2forms "$KIN/hydrogen-ignition-delay/Jachimowski-1992-species.inp" "$HERE/inputs/h2o2-rate-forms.lua"

# Sample data of the reference's unit tests (known-answer tests).
cp "$REF/src/kinetics/sample-input/H2-I2-HI.lua" "$OUT/h2i2-gas.lua"
cp "$REF/src/kinetics/sample-input/H2-I2-inp.lua" "$OUT/h2i2-chem.lua"
cp "$REF/src/kinetics/sample-input/N2-diss.lua" "$OUT/n2-diss-rate.lua"
cp "$REF/src/gas/sample-data/O-thermo.lua" "$OUT/O-thermo.lua"
cp "$REF/src/gas/sample-data/therm-perf-5-species-air.lua" "$OUT/tpg-air5-gas.lua"
cp "$REF/src/gas/sample-data/five-species-air.lua" "$OUT/air5-2T-gas.lua"   # two_temperature_gas.d:704-738
# The DRM19 example's comparison data (Eilmer3's fixed-volume reactor, CH4:O2:N2 = 1:2:7.52 at 2000 K
# and 1 atm, 2000 steps of 2e-7 s): time and temperature columns.
grep -v '^[A-Za-z#]' "$KIN/methane-combustion-w-drm19/eilmer3-result-for-comparison.data" | awk '{print $1, $4}' \
    > "$HERE/drm19-fvr-eilmer3-T.txt"
# The reference's Python binding (CFFI, dlopen("libgas.so")), unmodified, for the drop-in test of the C ABI
# (tests/test_gpu_ref_binding.py).
cp "$REF/src/lib/gdtk/gas.py" "$HERE/ref_gdtk/gdtk/gas.py"
chmod u+w "$OUT"/*.lua "$HERE/ref_gdtk/gdtk/gas.py"
echo "fixtures written to $OUT"
