species = {[0]='N2', [1]='O2', [2]='H2', [3]='H2O', [4]='OH', [5]='HO2', [6]='H2O2', [7]='NO', [8]='NO2', [9]='HNO', [10]='N', [11]='H', [12]='O', }
config = {
  tempLimits = {lower=300.000000, upper=50000.000000},
  odeStep = {method='alpha-qss', eps1= 1.000000e-03, eps2= 5.000000e-04, delta= 1.000000e-10, maxIters=10},
  tightTempCoupling = true,
  maxSubcycles = 10000,
  maxAttempts = 4
}

reaction = {}
reaction[1] = {
  equation = "H2 + O2 <=> H + HO2",
  type = "elementary",
  frc = {model='Arrhenius2', logA=1.806400580001e+01, B=0.000000000000e+00, C=2.860200000000e+04, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 1, 2,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 5, 11,},
  prodCoeffs = { 1, 1,},
  label = "r1",
}

reaction[2] = {
  equation = "H + O2 <=> OH + O",
  type = "elementary",
  frc = {model='Arrhenius2', logA=1.920913810432e+01, B=2.000000000000e-05, C=8.459740000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 1, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4, 12,},
  prodCoeffs = { 1, 1,},
  label = "r2",
}

reaction[3] = {
  equation = "O + H2 <=> OH + H",
  type = "elementary",
  frc = {model='Arrhenius', A=5.060000000000e-02, n=2.670000, C=3.167370000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 2, 12,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4, 11,},
  prodCoeffs = { 1, 1,},
  label = "r3",
}

reaction[4] = {
  equation = "OH + H2 <=> H2O + H",
  type = "elementary",
  frc = {model='Arrhenius', A=2.160000000000e+02, n=1.510000, C=1.727200000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 2, 4,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 3, 11,},
  prodCoeffs = { 1, 1,},
  label = "r4",
}

reaction[5] = {
  equation = "OH + OH <=> H2O + O",
  type = "elementary",
  frc = {model='Arrhenius', A=1.500000000000e+03, n=1.140000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4,},
  reacCoeffs = { 2,},
  prodIdx = { 3, 12,},
  prodCoeffs = { 1, 1,},
  label = "r5",
}

reaction[6] = {
  equation = "H + OH + M <=> H2O + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=8.620000000000e+09, n=-2.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 3,},
  prodCoeffs = { 1,},
  efficiencies = {
    [0]=1.000000e+00,
    [1]=1.000000e+00,
    [2]=2.500000e+00,
    [3]=1.600000e+01,
    [4]=1.000000e+00,
    [5]=1.000000e+00,
    [6]=1.000000e+00,
    [7]=1.000000e+00,
    [8]=1.000000e+00,
    [9]=1.000000e+00,
    [10]=1.000000e+00,
    [11]=1.000000e+00,
    [12]=1.000000e+00,
  },
  label = "r6",
}

reaction[7] = {
  equation = "H + H + M <=> H2 + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=7.300000000000e+05, n=-1.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 11,},
  reacCoeffs = { 2,},
  prodIdx = { 2,},
  prodCoeffs = { 1,},
  efficiencies = {
    [0]=1.000000e+00,
    [1]=1.000000e+00,
    [2]=2.500000e+00,
    [3]=1.600000e+01,
    [4]=1.000000e+00,
    [5]=1.000000e+00,
    [6]=1.000000e+00,
    [7]=1.000000e+00,
    [8]=1.000000e+00,
    [9]=1.000000e+00,
    [10]=1.000000e+00,
    [11]=1.000000e+00,
    [12]=1.000000e+00,
  },
  label = "r7",
}

reaction[8] = {
  equation = "HO2 + H <=> OH + OH",
  type = "elementary",
  frc = {model='Arrhenius2', logA=1.882614585206e+01, B=0.000000000000e+00, C=5.035560000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 5, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4,},
  prodCoeffs = { 2,},
  label = "r11",
}

reaction[9] = {
  equation = "HO2 + OH <=> H2O + O2",
  type = "elementary",
  frc = {model='Arrhenius', A=2.000000000000e+07, n=0.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4, 5,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 1, 3,},
  prodCoeffs = { 1, 1,},
  label = "r13",
}

reaction[10] = {
  equation = "H + O2 (+ M) <=> HO2 (+ M)",
  type = "elementary",
  frc = {model='Lindemann-Hinshelwood',
   kInf={A=5.590000000000e+07, n=0.200000, C=0.000000000000e+00, rctIndex=-1},
   k0={A=2.650000000000e+07, n=-1.300000, C=0.000000000000e+00, rctIndex=-1}
},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 1, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 5,},
  prodCoeffs = { 1,},
  efficiencies = {
    [0]=1.000000e+00,
    [1]=1.000000e+00,
    [2]=2.500000e+00,
    [3]=1.600000e+01,
    [4]=1.000000e+00,
    [5]=1.000000e+00,
    [6]=1.200000e+01,
    [7]=1.000000e+00,
    [8]=1.000000e+00,
    [9]=1.000000e+00,
    [10]=1.000000e+00,
    [11]=1.000000e+00,
    [12]=1.000000e+00,
  },
  label = "lh",
}

reaction[11] = {
  equation = "H2O2 (+ M) <=> 2OH (+ M)",
  type = "elementary",
  frc = {model='Yungster-Rabinowitz',
   kInf={A=8.590000000000e+14, n=0.000000, C=2.443639291465e+04, rctIndex=-1},
   k0={A=9.550000000000e+09, n=0.000000, C=2.123741948470e+04, rctIndex=-1},
 c=1.756000000000e+03,  a=7.350000000000e-01,  b=9.400000000000e+01, 
},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 6,},
  reacCoeffs = { 1,},
  prodIdx = { 4,},
  prodCoeffs = { 2,},
  efficiencies = {
    [0]=1.500000e+00,
    [1]=1.000000e+00,
    [2]=2.500000e+00,
    [3]=1.500000e+01,
    [4]=1.000000e+00,
    [5]=1.000000e+00,
    [6]=1.500000e+01,
    [7]=1.000000e+00,
    [8]=1.000000e+00,
    [9]=1.000000e+00,
    [10]=1.000000e+00,
    [11]=1.000000e+00,
    [12]=1.000000e+00,
  },
  label = "yr",
}

