-- H2 + I2 <=> 2 HI with the rate constant the reference's unit tests build in code
-- (src/kinetics/reaction_mechanism.d:264-283 and src/kinetics/reaction.d:538-556):
-- ArrheniusRateConstant(1.94e14, 0.0, 20620.0) used unscaled for both directions.
species = {[0]='H2', [1]='I2', [2]='HI', }
config = {
  maxSubcycles = 50,
  maxAttempts = 2,
  tightTempCoupling = false,
  tempLimits = {lower=100.000000, upper=10000.000000},
  odeStep = {method='rkf', errTol=1.0e-3},
}
reaction = {}
reaction[1] = {
  equation = "H2 + I2 <=> 2 HI",
  type = "elementary",
  frc = {model='Arrhenius', A=1.94e14, n=0.000000, C=2.062e4, rctIndex=-1 },
  brc = {model='Arrhenius', A=1.94e14, n=0.000000, C=2.062e4, rctIndex=-1 },
  ec = {},
  reacIdx = { 0, 1,},
  reacCoeffs = { 1, 1,},
  prodIdx = { 2,},
  prodCoeffs = { 2,},
}
