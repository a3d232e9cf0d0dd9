species = {[0]='N2', [1]='O2', [2]='N', [3]='O', [4]='NO', }
config = {
  tempLimits = {lower=300.000000, upper=50000.000000},
  odeStep = {method='rkf', errTol=1.000000e-03},
  tightTempCoupling = false,
  maxSubcycles = 10000,
  maxAttempts = 4
}

reaction = {}
reaction[1] = {
  equation = "N2 + M <=> N + N + M",
  type = "anonymous_collider",
  frc = {model='Marrone-Treanor', T_D=1.137001623669e+05, U=3.790005412232e+04, theta=3.393440000000e+03, mode=0, rate={model='Arrhenius', A=7.000000000000e+15, n=-1.600000, C=1.132000000000e+05, rctIndex=-1}},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 0,},
  reacCoeffs = { 1,},
  prodIdx = { 2,},
  prodCoeffs = { 2,},
  efficiencies = {
    [0]=1.000000e+00,
    [1]=1.000000e+00,
    [2]=4.285700e+00,
    [3]=4.285700e+00,
    [4]=1.000000e+00,
  },
  label = "r1",
}

reaction[2] = {
  equation = "O2 + M <=> O + O + M",
  type = "anonymous_collider",
  frc = {model='Modified-Marrone-Treanor', T_D=5.993745937819e+04, aU=1.500000000000e-01, Ustar=4.000000000000e+04, theta=2.273540000000e+03, mode=0, rate={model='Park', A=2.000000000000e+15, n=-1.500000, C=5.950000000000e+04, s=0.500000, mode=0 }, non_boltzmann_correction = {model='constant', factor=0.900000}},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 1,},
  reacCoeffs = { 1,},
  prodIdx = { 3,},
  prodCoeffs = { 2,},
  efficiencies = {
    [0]=1.000000e+00,
    [1]=1.000000e+00,
    [2]=5.000000e+00,
    [3]=5.000000e+00,
    [4]=1.000000e+00,
  },
  label = "r2",
}

reaction[3] = {
  equation = "NO + M <=> N + O + M",
  type = "anonymous_collider",
  frc = {model='Park', A=5.000000000000e+09, n=0.000000, C=7.550000000000e+04, s=0.500000, mode=0 },
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4,},
  reacCoeffs = { 1,},
  prodIdx = { 2, 3,},
  prodCoeffs = { 1, 1,},
  efficiencies = {
    [0]=1.000000e+00,
    [1]=1.000000e+00,
    [2]=2.000000e+01,
    [3]=2.000000e+01,
    [4]=1.000000e+00,
  },
  label = "r3",
}

reaction[4] = {
  equation = "NO + O <=> O2 + N",
  type = "elementary",
  frc = {model='Arrhenius', A=8.400000000000e+06, n=0.000000, C=1.945000000000e+04, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 3, 4,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 1, 2,},
  prodCoeffs = { 1, 1,},
  label = "r4",
}

reaction[5] = {
  equation = "N2 + O <=> NO + N",
  type = "elementary",
  frc = {model='Arrhenius', A=6.400000000000e+11, n=-1.000000, C=3.840000000000e+04, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 0, 3,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 2, 4,},
  prodCoeffs = { 1, 1,},
  label = "r5",
}

