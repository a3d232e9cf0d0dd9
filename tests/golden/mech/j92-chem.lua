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

reaction[2] = {
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

reaction[3] = {
  equation = "H + O + M <=> OH + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=2.600000000000e+04, n=-0.600000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 11, 12,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4,},
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
  label = "r8",
}

reaction[4] = {
  equation = "O + O + M <=> O2 + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=1.100000000000e+05, n=-1.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 12,},
  reacCoeffs = { 2,},
  prodIdx = { 1,},
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
  label = "r9",
}

reaction[5] = {
  equation = "H + O2 + M <=> HO2 + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=2.300000000000e+06, n=-1.000000, C=0.000000000000e+00, rctIndex=-1},
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
    [6]=1.000000e+00,
    [7]=1.000000e+00,
    [8]=1.000000e+00,
    [9]=1.000000e+00,
    [10]=1.000000e+00,
    [11]=1.000000e+00,
    [12]=1.000000e+00,
  },
  label = "r10",
}

reaction[6] = {
  equation = "OH + OH + M <=> H2O2 + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=1.600000000000e+10, n=-2.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4,},
  reacCoeffs = { 2,},
  prodIdx = { 6,},
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
  label = "r19",
}

reaction[7] = {
  equation = "N + N + M <=> N2 + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=2.800000000000e+05, n=-0.800000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 10,},
  reacCoeffs = { 2,},
  prodIdx = { 0,},
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
  label = "r20",
}

reaction[8] = {
  equation = "H + NO + M <=> HNO + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=5.400000000000e+03, n=0.000000, C=-3.021330000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 7, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 9,},
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
  label = "r24",
}

reaction[9] = {
  equation = "M + NO2 <=> NO + O + M",
  type = "anonymous_collider",
  frc = {model='Arrhenius', A=1.160000000000e+10, n=0.000000, C=3.323470000000e+04, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 8,},
  reacCoeffs = { 1,},
  prodIdx = { 7, 12,},
  prodCoeffs = { 1, 1,},
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
  label = "r33",
}

reaction[10] = {
  equation = "H2 + O2 <=> H + HO2",
  type = "elementary",
  frc = {model='Arrhenius', A=7.000000000000e+07, n=0.000000, C=2.860200000000e+04, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 1, 2,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 5, 11,},
  prodCoeffs = { 1, 1,},
  label = "r1",
}

reaction[11] = {
  equation = "H + O2 <=> OH + O",
  type = "elementary",
  frc = {model='Arrhenius', A=2.200000000000e+08, n=0.000000, C=8.459740000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 1, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4, 12,},
  prodCoeffs = { 1, 1,},
  label = "r2",
}

reaction[12] = {
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

reaction[13] = {
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

reaction[14] = {
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

reaction[15] = {
  equation = "HO2 + H <=> OH + OH",
  type = "elementary",
  frc = {model='Arrhenius', A=1.500000000000e+08, n=0.000000, C=5.035560000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 5, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4,},
  prodCoeffs = { 2,},
  label = "r11",
}

reaction[16] = {
  equation = "HO2 + O <=> O2 + OH",
  type = "elementary",
  frc = {model='Arrhenius', A=2.000000000000e+07, n=0.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 5, 12,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 1, 4,},
  prodCoeffs = { 1, 1,},
  label = "r12",
}

reaction[17] = {
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

reaction[18] = {
  equation = "HO2 + HO2 <=> H2O2 + O2",
  type = "elementary",
  frc = {model='Arrhenius', A=2.000000000000e+06, n=0.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 5,},
  reacCoeffs = { 2,},
  prodIdx = { 1, 6,},
  prodCoeffs = { 1, 1,},
  label = "r14",
}

reaction[19] = {
  equation = "H + H2O2 <=> H2 + HO2",
  type = "elementary",
  frc = {model='Arrhenius', A=1.700000000000e+06, n=0.000000, C=1.903440000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 6, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 2, 5,},
  prodCoeffs = { 1, 1,},
  label = "r15",
}

reaction[20] = {
  equation = "H + H2O2 <=> OH + H2O",
  type = "elementary",
  frc = {model='Arrhenius', A=1.000000000000e+07, n=0.000000, C=1.802730000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 6, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 3, 4,},
  prodCoeffs = { 1, 1,},
  label = "r16",
}

reaction[21] = {
  equation = "O + H2O2 <=> OH + HO2",
  type = "elementary",
  frc = {model='Arrhenius', A=2.800000000000e+07, n=0.000000, C=3.222760000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 6, 12,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4, 5,},
  prodCoeffs = { 1, 1,},
  label = "r17",
}

reaction[22] = {
  equation = "OH + H2O2 <=> H2O + HO2",
  type = "elementary",
  frc = {model='Arrhenius', A=7.000000000000e+06, n=0.000000, C=7.226020000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4, 6,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 3, 5,},
  prodCoeffs = { 1, 1,},
  label = "r18",
}

reaction[23] = {
  equation = "N + O2 <=> NO + O",
  type = "elementary",
  frc = {model='Arrhenius', A=6.400000000000e+03, n=1.000000, C=3.172400000000e+03, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 1, 10,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 7, 12,},
  prodCoeffs = { 1, 1,},
  label = "r21",
}

reaction[24] = {
  equation = "N + NO <=> N2 + O",
  type = "elementary",
  frc = {model='Arrhenius', A=1.600000000000e+07, n=0.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 7, 10,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 0, 12,},
  prodCoeffs = { 1, 1,},
  label = "r22",
}

reaction[25] = {
  equation = "N + OH <=> NO + H",
  type = "elementary",
  frc = {model='Arrhenius', A=6.300000000000e+05, n=0.500000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4, 10,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 7, 11,},
  prodCoeffs = { 1, 1,},
  label = "r23",
}

reaction[26] = {
  equation = "H + HNO <=> NO + H2",
  type = "elementary",
  frc = {model='Arrhenius', A=4.800000000000e+06, n=0.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 9, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 2, 7,},
  prodCoeffs = { 1, 1,},
  label = "r25",
}

reaction[27] = {
  equation = "O + HNO <=> NO + OH",
  type = "elementary",
  frc = {model='Arrhenius', A=5.000000000000e+05, n=0.500000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 9, 12,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4, 7,},
  prodCoeffs = { 1, 1,},
  label = "r26",
}

reaction[28] = {
  equation = "OH + HNO <=> NO + H2O",
  type = "elementary",
  frc = {model='Arrhenius', A=3.600000000000e+07, n=0.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 4, 9,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 3, 7,},
  prodCoeffs = { 1, 1,},
  label = "r27",
}

reaction[29] = {
  equation = "HO2 + HNO <=> NO + H2O2",
  type = "elementary",
  frc = {model='Arrhenius', A=2.000000000000e+06, n=0.000000, C=0.000000000000e+00, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 5, 9,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 6, 7,},
  prodCoeffs = { 1, 1,},
  label = "r28",
}

reaction[30] = {
  equation = "HO2 + NO <=> NO2 + OH",
  type = "elementary",
  frc = {model='Arrhenius', A=3.400000000000e+06, n=0.000000, C=-1.309240000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 5, 7,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4, 8,},
  prodCoeffs = { 1, 1,},
  label = "r29",
}

reaction[31] = {
  equation = "HO2 + NO <=> HNO + O2",
  type = "elementary",
  frc = {model='Arrhenius', A=2.000000000000e+05, n=0.000000, C=5.035560000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 5, 7,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 1, 9,},
  prodCoeffs = { 1, 1,},
  label = "r30",
}

reaction[32] = {
  equation = "H + NO2 <=> NO + OH",
  type = "elementary",
  frc = {model='Arrhenius', A=3.500000000000e+08, n=0.000000, C=7.553340000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 8, 11,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 4, 7,},
  prodCoeffs = { 1, 1,},
  label = "r31",
}

reaction[33] = {
  equation = "O + NO2 <=> NO + O2",
  type = "elementary",
  frc = {model='Arrhenius', A=1.000000000000e+07, n=0.000000, C=3.021330000000e+02, rctIndex=-1},
  brc = {model='fromEqConst', rctIndex=-1},
  ec = {},
  reacIdx = { 8, 12,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 1, 7,},
  prodCoeffs = { 1, 1,},
  label = "r32",
}

