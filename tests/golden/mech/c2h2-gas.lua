
model = 'CompositeGas'
species = {'H2', 'H', 'O', 'O2', 'OH', 'H2O', 'HO2', 'H2O2', 'C', 'CH', 'CH2', 'CH2', 'CH3', 'CH4', 'CO', 'CO2', 'HCO', 'CH2O', 'CH2OH', 'CH3O', 'CH3OH', 'C2H', 'C2H2', 'H2CC', 'C2H3', 'C2H4', 'C2H5', 'C2H6', 'HCCO', 'CH2CO', 'HCCOH', 'C2O', 'CH2CHO', 'CH3CHO', 'CH3CO', 'C3H2', 'C3H3', 'pC3H4', 'aC3H4', 'cC3H4', 'aC3H5', 'CH3CCH2', 'CH3CHCH', 'C3H6', 'C2H3CHO', 'nC3H7', 'iC3H7', 'C3H8', 'C4H', 'C4H2', 'H2C4O', 'n-C4H3', 'i-C4H3', 'C4H4', 'n-C4H5', 'i-C4H5', 'C4H6', 'C4H612', 'C4H7', 'C4H81', 'C6H2', 'C6H3', 'l-C6H4', 'c-C6H4', 'A1', 'A1-', 'C6H5O', 'C6H5OH', 'C5H6', 'C5H5', 'C5H4O', 'C5H4OH', 'C5H5O', 'Ar', 'N2', }

physical_model = 'thermally-perfect-gas'
energyModes = {'equilibrium'}
db = {}
db['H2'] = {}
db['H2'].atomicConstituents = { H=2, }
db['H2'].charge = 0
db['H2'].M = 2.01588000e-03
db['H2'].sigma = 2.92000000
db['H2'].epsilon = 38.00000000
db['H2'].Lewis = 0.31700000
db['H2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.344331120e+00,
    7.980520750e-03,
   -1.947815100e-05,
    2.015720940e-08,
   -7.376117610e-12,
   -9.179351730e+02,
    6.830102380e-01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.337279200e+00,
   -4.940247310e-05,
    4.994567780e-07,
   -1.795663940e-10,
    2.002553760e-14,
   -9.501589220e+02,
   -3.205023310e+00,
  },
}
db['H2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  7.4553182e-01,
      B =  4.3555109e+01,
      C = -3.2579340e+03,
      D =  1.3556243e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  9.6730605e-01,
      B =  6.7931897e+02,
      C = -2.1025179e+05,
      D = -1.8251697e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  1.0126129e+00,
      B =  1.4973739e+03,
      C = -1.4428484e+06,
      D = -2.3254928e+00,
   },
}
db['H2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  1.0059461e+00,
      B =  2.7951262e+02,
      C = -2.9792018e+04,
      D =  1.1996252e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  1.0582450e+00,
      B =  2.4875372e+02,
      C =  1.1736907e+04,
      D =  8.2758695e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A = -2.2364420e-01,
      B = -6.9650442e+03,
      C = -7.7771313e+04,
      D =  1.3189369e+01,
   },
}
db['H'] = {}
db['H'].atomicConstituents = { H=1, }
db['H'].charge = 0
db['H'].M = 1.00794000e-03
db['H'].sigma = 2.05000000
db['H'].epsilon = 145.00000000
db['H'].Lewis = 0.18900000
db['H'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.500000000e+00,
    7.053328190e-13,
   -1.995919640e-15,
    2.300816320e-18,
   -9.277323320e-22,
    2.547365990e+04,
   -4.466828530e-01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.500000010e+00,
   -2.308429730e-11,
    1.615619480e-14,
   -4.735152350e-18,
    4.981973570e-22,
    2.547365990e+04,
   -4.466829140e-01,
  },
}
db['H'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  7.4226149e-01,
      B = -4.0132865e+02,
      C =  1.8554165e+05,
      D =  4.6741844e-02,
   },
   segment1 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.7486623e-01,
      B = -2.5022902e+03,
      C =  7.0955048e+06,
      D = -9.3888455e-01,
   },
}
db['H'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  7.4166119e-01,
      B = -4.0487203e+02,
      C =  1.8775642e+05,
      D =  3.4843121e+00,
   },
   segment1 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.7447639e-01,
      B = -2.5089452e+03,
      C =  7.1081294e+06,
      D =  2.4970991e+00,
   },
}
db['O'] = {}
db['O'].atomicConstituents = { O=1, }
db['O'].charge = 0
db['O'].M = 1.59994000e-02
db['O'].sigma = 2.75000000
db['O'].epsilon = 80.00000000
db['O'].Lewis = 0.71200000
db['O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.168267100e+00,
   -3.279318840e-03,
    6.643063960e-06,
   -6.128066240e-09,
    2.112659710e-12,
    2.912225920e+04,
    2.051933460e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.569420780e+00,
   -8.597411370e-05,
    4.194845890e-08,
   -1.001777990e-11,
    1.228336910e-15,
    2.921757910e+04,
    4.784338640e+00,
  },
}
db['O'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  7.7269241e-01,
      B =  8.3842977e+01,
      C = -5.8502098e+04,
      D =  8.5100827e-01,
   },
   segment1 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.7669586e-01,
      B =  1.0158420e+03,
      C = -1.0884566e+06,
      D = -1.8001077e-01,
   },
}
db['O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  7.7271664e-01,
      B =  8.3989100e+01,
      C = -5.8580966e+04,
      D =  1.5179900e+00,
   },
   segment1 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.7676666e-01,
      B =  1.0170744e+03,
      C = -1.0906690e+06,
      D =  4.8644232e-01,
   },
}
db['O2'] = {}
db['O2'].atomicConstituents = { O=2, }
db['O2'].charge = 0
db['O2'].M = 3.19988000e-02
db['O2'].sigma = 3.45800000
db['O2'].epsilon = 107.40000000
db['O2'].Lewis = 1.08600000
db['O2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.782456360e+00,
   -2.996734160e-03,
    9.847302010e-06,
   -9.681295090e-09,
    3.243728370e-12,
   -1.063943560e+03,
    3.657675730e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.282537840e+00,
    1.483087540e-03,
   -7.579666690e-07,
    2.094705550e-10,
   -2.167177940e-14,
   -1.088457720e+03,
    5.453231290e+00,
  },
}
db['O2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.0916180e-01,
      B = -5.2244847e+01,
      C = -5.9974009e+02,
      D =  2.0410801e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  7.2216486e-01,
      B =  1.7550839e+02,
      C = -5.7974816e+04,
      D =  1.0901044e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  7.3981127e-01,
      B =  3.9194906e+02,
      C = -3.7833168e+05,
      D =  9.0931780e-01,
   },
}
db['O2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  7.7229167e-01,
      B =  6.8463210e+00,
      C = -5.8933377e+03,
      D =  1.2210365e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  9.0917351e-01,
      B =  2.9124182e+02,
      C = -7.9650171e+04,
      D =  6.4851631e-02,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A = -1.1218262e+00,
      B = -1.9286378e+04,
      C =  2.3295011e+07,
      D =  2.0342043e+01,
   },
}
db['OH'] = {}
db['OH'].atomicConstituents = { H=1, O=1, }
db['OH'].charge = 0
db['OH'].M = 1.70073400e-02
db['OH'].sigma = 2.75000000
db['OH'].epsilon = 80.00000000
db['OH'].Lewis = 0.73600000
db['OH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.992015430e+00,
   -2.401317520e-03,
    4.617938410e-06,
   -3.881133330e-09,
    1.364114700e-12,
    3.615080560e+03,
   -1.039254580e-01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.092887670e+00,
    5.484297160e-04,
    1.265052280e-07,
   -8.794615560e-11,
    1.174123760e-14,
    3.858657000e+03,
    4.476696100e+00,
  },
}
db['OH'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  5.9711536e-01,
      B = -4.6100678e+02,
      C =  3.7606286e+04,
      D =  2.4041761e+00,
   },
   segment1 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  6.4287721e-01,
      B = -1.8173747e+02,
      C = -8.8543767e+04,
      D =  1.9636057e+00,
   },
}
db['OH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.8627561e-01,
      B = -7.4033274e+02,
      C =  2.7559033e+04,
      D =  2.8308741e+00,
   },
   segment1 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A = -4.7918112e-01,
      B = -9.3769908e+03,
      C =  7.0509952e+06,
      D =  1.4203688e+01,
   },
}
db['H2O'] = {}
db['H2O'].atomicConstituents = { H=2, O=1, }
db['H2O'].charge = 0
db['H2O'].M = 1.80152800e-02
db['H2O'].sigma = 2.60500000
db['H2O'].epsilon = 572.40000000
db['H2O'].Lewis = 0.85400000
db['H2O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.198640560e+00,
   -2.036434100e-03,
    6.520402110e-06,
   -5.487970620e-09,
    1.771978170e-12,
   -3.029372670e+04,
   -8.490322080e-01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.033992490e+00,
    2.176918040e-03,
   -1.640725180e-07,
   -9.704198700e-11,
    1.682009920e-14,
   -3.000429710e+04,
    4.966770100e+00,
  },
}
db['H2O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 373.2,
      T_upper = 1073.2,
      A =  5.0019557e-01,
      B = -6.9712796e+02,
      C =  8.8163892e+04,
      D =  3.0836508e+00,
   },
   segment1 = {
      T_lower = 1073.2,
      T_upper = 5000.0,
      A =  5.8988538e-01,
      B = -5.3769814e+02,
      C =  5.4263513e+04,
      D =  2.3386375e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  6.4330087e-01,
      B = -9.5668913e+01,
      C = -3.7742283e+05,
      D =  1.8125190e+00,
   },
}
db['H2O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 373.2,
      T_upper = 1073.2,
      A =  1.0966389e+00,
      B = -5.5513429e+02,
      C =  1.0623408e+05,
      D = -2.4664550e-01,
   },
   segment1 = {
      T_lower = 1073.2,
      T_upper = 5000.0,
      A =  3.9367933e-01,
      B = -2.2524226e+03,
      C =  6.1217458e+05,
      D =  5.8011317e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A = -4.1858737e-01,
      B = -1.4096649e+04,
      C =  1.9179190e+07,
      D =  1.4345613e+01,
   },
}
db['HO2'] = {}
db['HO2'].atomicConstituents = { H=1, O=2, }
db['HO2'].charge = 0
db['HO2'].M = 3.30067400e-02
db['HO2'].sigma = 3.45800000
db['HO2'].epsilon = 107.40000000
db['HO2'].Lewis = 1.07900000
db['HO2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.301798010e+00,
   -4.749120510e-03,
    2.115828910e-05,
   -2.427638940e-08,
    9.292251240e-12,
    2.948080400e+02,
    3.716662450e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.017210900e+00,
    2.239820130e-03,
   -6.336581500e-07,
    1.142463700e-10,
   -1.079085350e-14,
    1.118567130e+02,
    3.785102150e+00,
  },
}
db['HO2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['HO2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['H2O2'] = {}
db['H2O2'].atomicConstituents = { H=2, O=2, }
db['H2O2'].charge = 0
db['H2O2'].M = 3.40146800e-02
db['H2O2'].sigma = 3.45800000
db['H2O2'].epsilon = 107.40000000
db['H2O2'].Lewis = 1.15200000
db['H2O2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.276112690e+00,
   -5.428224170e-04,
    1.673357010e-05,
   -2.157708130e-08,
    8.624543630e-12,
   -1.770258210e+04,
    3.435050740e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.165002850e+00,
    4.908316940e-03,
   -1.901392250e-06,
    3.711859860e-10,
   -2.879083050e-14,
   -1.786178770e+04,
    2.916156620e+00,
  },
}
db['H2O2'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  9.9686871e-01,
      B = -4.1461068e+01,
      C =  8.7172900e+03,
      D = -1.5770256e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  5.7419481e-01,
      B = -5.0408983e+02,
      C =  4.8898234e+04,
      D =  1.7621537e+00,
   },
}
db['H2O2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  1.1075595e+00,
      B = -2.0746382e+02,
      C =  2.3930396e+04,
      D = -1.2685243e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  4.6981213e-01,
      B = -1.1937657e+03,
      C =  2.2076993e+05,
      D =  3.9203830e+00,
   },
}
db['C'] = {}
db['C'].atomicConstituents = { C=1, }
db['C'].charge = 0
db['C'].M = 1.20107000e-02
db['C'].sigma = 3.29800000
db['C'].epsilon = 71.40000000
db['C'].Lewis = 1.15200000
db['C'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.554239550e+00,
   -3.215377240e-04,
    7.337922450e-07,
   -7.322348890e-10,
    2.665214460e-13,
    8.544388320e+04,
    4.531308480e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.492668880e+00,
    4.798892840e-05,
   -7.243350200e-08,
    3.742910290e-11,
   -4.872778930e-15,
    8.545129530e+04,
    4.801503730e+00,
  },
}
db['C'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH'] = {}
db['CH'].atomicConstituents = { H=1, C=1, }
db['CH'].charge = 0
db['CH'].M = 1.30186400e-02
db['CH'].sigma = 2.75000000
db['CH'].epsilon = 80.00000000
db['CH'].Lewis = 1.15200000
db['CH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.489816650e+00,
    3.238355410e-04,
   -1.688990650e-06,
    3.162173270e-09,
   -1.406090670e-12,
    7.079729340e+04,
    2.084011080e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.878464730e+00,
    9.709136810e-04,
    1.444456550e-07,
   -1.306878490e-10,
    1.760793830e-14,
    7.101243640e+04,
    5.484979990e+00,
  },
}
db['CH'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  6.3306702e-01,
      B = -7.5491296e+00,
      C = -2.1396736e+03,
      D =  1.4781500e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.4807346e-01,
      B =  3.1141665e+00,
      C = -1.8292566e+03,
      D =  1.3638041e+00,
   },
}
db['CH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  1.0884807e+00,
      B =  2.7220319e+02,
      C = -2.2480091e+04,
      D = -6.4679028e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  4.4721563e-01,
      B = -1.0513211e+03,
      C =  2.8092259e+05,
      D =  4.8038688e+00,
   },
}
db['CH2'] = {}
db['CH2'].atomicConstituents = { H=2, C=1, }
db['CH2'].charge = 0
db['CH2'].M = 1.40265800e-02
db['CH2'].sigma = 3.80000000
db['CH2'].epsilon = 144.00000000
db['CH2'].Lewis = 1.02300000
db['CH2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.762678670e+00,
    9.688721430e-04,
    2.794898410e-06,
   -3.850911530e-09,
    1.687417190e-12,
    4.600404010e+04,
    1.562531850e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.874101130e+00,
    3.656392920e-03,
   -1.408945970e-06,
    2.601795490e-10,
   -1.877275670e-14,
    4.626360400e+04,
    6.171193240e+00,
  },
}
db['CH2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH2'] = {}
db['CH2'].atomicConstituents = { H=2, C=1, }
db['CH2'].charge = 0
db['CH2'].M = 1.40265800e-02
db['CH2'].sigma = 3.80000000
db['CH2'].epsilon = 144.00000000
db['CH2'].Lewis = 1.02300000
db['CH2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.762678670e+00,
    9.688721430e-04,
    2.794898410e-06,
   -3.850911530e-09,
    1.687417190e-12,
    4.600404010e+04,
    1.562531850e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.874101130e+00,
    3.656392920e-03,
   -1.408945970e-06,
    2.601795490e-10,
   -1.877275670e-14,
    4.626360400e+04,
    6.171193240e+00,
  },
}
db['CH2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH3'] = {}
db['CH3'].atomicConstituents = { H=3, C=1, }
db['CH3'].charge = 0
db['CH3'].M = 1.50345200e-02
db['CH3'].sigma = 3.80000000
db['CH3'].epsilon = 144.00000000
db['CH3'].Lewis = 1.04900000
db['CH3'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.673590400e+00,
    2.010951750e-03,
    5.730218560e-06,
   -6.871174250e-09,
    2.543857340e-12,
    1.644499880e+04,
    1.604564330e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.285717720e+00,
    7.239900370e-03,
   -2.987143480e-06,
    5.956846440e-10,
   -4.671543940e-14,
    1.677558430e+04,
    8.480071790e+00,
  },
}
db['CH3'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH3'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH4'] = {}
db['CH4'].atomicConstituents = { H=4, C=1, }
db['CH4'].charge = 0
db['CH4'].M = 1.60424600e-02
db['CH4'].sigma = 3.74600000
db['CH4'].epsilon = 141.40000000
db['CH4'].Lewis = 1.04300000
db['CH4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    5.149876130e+00,
   -1.367097880e-02,
    4.918005990e-05,
   -4.847430260e-08,
    1.666939560e-11,
   -1.024664760e+04,
   -4.641303760e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    7.485149500e-02,
    1.339094670e-02,
   -5.732858090e-06,
    1.222925350e-09,
   -1.018152300e-13,
   -9.468344590e+03,
    1.843731800e+01,
  },
}
db['CH4'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  5.7643622e-01,
      B = -9.3704079e+01,
      C =  8.6992395e+02,
      D =  1.7333347e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.6400044e-01,
      B =  1.0860843e+01,
      C = -7.6307841e+03,
      D =  1.0323984e+00,
   },
}
db['CH4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  1.0238177e+00,
      B = -3.1092375e+02,
      C =  3.2944309e+04,
      D =  6.7787437e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  7.7485028e-01,
      B = -4.0089627e+02,
      C = -4.6551082e+04,
      D =  2.5671481e+00,
   },
}
db['CO'] = {}
db['CO'].atomicConstituents = { O=1, C=1, }
db['CO'].charge = 0
db['CO'].M = 2.80101000e-02
db['CO'].sigma = 3.65000000
db['CO'].epsilon = 98.10000000
db['CO'].Lewis = 1.17100000
db['CO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.579533470e+00,
   -6.103536800e-04,
    1.016814330e-06,
    9.070058840e-10,
   -9.044244990e-13,
   -1.434408600e+04,
    3.508409280e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.715185610e+00,
    2.062527430e-03,
   -9.988257710e-07,
    2.300530080e-10,
   -2.036477160e-14,
   -1.415187240e+04,
    7.818687720e+00,
  },
}
db['CO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4175411e+00,
      B =  8.0462671e+03,
      C =  3.1090740e+06,
      D = -1.4516932e+01,
   },
}
db['CO2'] = {}
db['CO2'].atomicConstituents = { O=2, C=1, }
db['CO2'].charge = 0
db['CO2'].M = 4.40100000e-02
db['CO2'].sigma = 3.76300000
db['CO2'].epsilon = 244.00000000
db['CO2'].Lewis = 1.40400000
db['CO2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.356773520e+00,
    8.984596770e-03,
   -7.123562690e-06,
    2.459190220e-09,
   -1.436995480e-13,
   -4.837196970e+04,
    9.901052220e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.857460290e+00,
    4.414370260e-03,
   -2.214814040e-06,
    5.234901880e-10,
   -4.720841640e-14,
   -4.875916600e+04,
    2.271638060e+00,
  },
}
db['CO2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  5.1137258e-01,
      B = -2.2951321e+02,
      C =  1.3710678e+04,
      D =  2.7075538e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.3978285e-01,
      B = -4.2637076e+01,
      C = -1.5522605e+04,
      D =  1.6628843e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  7.2150912e-01,
      B =  7.5012895e+02,
      C = -1.1825507e+06,
      D =  8.5493645e-01,
   },
}
db['CO2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  4.8056568e-01,
      B = -5.0786720e+02,
      C =  3.5088811e+04,
      D =  3.6747794e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.9857277e-01,
      B = -1.1830477e+02,
      C = -5.0688859e+04,
      D =  1.8650551e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  1.0518358e+00,
      B = -4.2555944e+03,
      C =  1.4288688e+07,
      D = -8.8950473e-01,
   },
}
db['HCO'] = {}
db['HCO'].atomicConstituents = { H=1, O=1, C=1, }
db['HCO'].charge = 0
db['HCO'].M = 2.90180400e-02
db['HCO'].sigma = 3.59000000
db['HCO'].epsilon = 498.00000000
db['HCO'].Lewis = 1.15200000
db['HCO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.221185840e+00,
   -3.243925320e-03,
    1.377994460e-05,
   -1.331440930e-08,
    4.337688650e-12,
    3.839564960e+03,
    3.394372430e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.772174380e+00,
    4.956955260e-03,
   -2.484456130e-06,
    5.891617780e-10,
   -5.335087110e-14,
    4.011918150e+03,
    9.798344920e+00,
  },
}
db['HCO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['HCO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH2O'] = {}
db['CH2O'].atomicConstituents = { H=2, O=1, C=1, }
db['CH2O'].charge = 0
db['CH2O'].M = 3.00259800e-02
db['CH2O'].sigma = 3.59000000
db['CH2O'].epsilon = 498.00000000
db['CH2O'].Lewis = 1.32900000
db['CH2O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.793723150e+00,
   -9.908333690e-03,
    3.732200080e-05,
   -3.792852610e-08,
    1.317726520e-11,
   -1.430895670e+04,
    6.028129000e-01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.760690080e+00,
    9.200000820e-03,
   -4.422588130e-06,
    1.006412120e-09,
   -8.838556400e-14,
   -1.399583230e+04,
    1.365632300e+01,
  },
}
db['CH2O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH2O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH2OH'] = {}
db['CH2OH'].atomicConstituents = { H=3, O=1, C=1, }
db['CH2OH'].charge = 0
db['CH2OH'].M = 3.10339200e-02
db['CH2OH'].sigma = 3.69000000
db['CH2OH'].epsilon = 417.00000000
db['CH2OH'].Lewis = 1.15200000
db['CH2OH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.863889180e+00,
    5.596723040e-03,
    5.932717910e-06,
   -1.045320120e-08,
    4.369672780e-12,
   -3.193913670e+03,
    5.473022430e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.692665690e+00,
    8.645767970e-03,
   -3.751011200e-06,
    7.872346360e-10,
   -6.485542010e-14,
   -3.242506270e+03,
    5.810432150e+00,
  },
}
db['CH2OH'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH2OH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH3O'] = {}
db['CH3O'].atomicConstituents = { H=3, O=1, C=1, }
db['CH3O'].charge = 0
db['CH3O'].M = 3.10339200e-02
db['CH3O'].sigma = 3.69000000
db['CH3O'].epsilon = 417.00000000
db['CH3O'].Lewis = 1.36000000
db['CH3O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.106204000e+00,
    7.216595000e-03,
    5.338472000e-06,
   -7.377636000e-09,
    2.075610000e-12,
    9.786011000e+02,
    1.315217700e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.770799000e+00,
    7.871497000e-03,
   -2.656384000e-06,
    3.944431000e-10,
   -2.112616000e-14,
    1.278325200e+02,
    2.929575000e+00,
  },
}
db['CH3O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH3O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH3OH'] = {}
db['CH3OH'].atomicConstituents = { H=4, O=1, C=1, }
db['CH3OH'].charge = 0
db['CH3OH'].M = 3.20418600e-02
db['CH3OH'].sigma = 3.62600000
db['CH3OH'].epsilon = 481.80000000
db['CH3OH'].Lewis = 1.15200000
db['CH3OH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    5.715395820e+00,
   -1.523091290e-02,
    6.524411550e-05,
   -7.108068890e-08,
    2.613526980e-11,
   -2.564276560e+04,
   -1.504098230e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.789707910e+00,
    1.409382920e-02,
   -6.365008350e-06,
    1.381710850e-09,
   -1.170602200e-13,
   -2.537487470e+04,
    1.450236230e+01,
  },
}
db['CH3OH'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH3OH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C2H'] = {}
db['C2H'].atomicConstituents = { H=1, Ar=0, N=0, O=0, He=0, C=2, }
db['C2H'].charge = 0
db['C2H'].M = 2.50290000e-02
db['C2H'].sigma = 4.10000000
db['C2H'].epsilon = 209.00000000
db['C2H'].Lewis = 1.15200000
db['C2H'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.889657330e+00,
    1.340996110e-02,
   -2.847695010e-05,
    2.947910450e-08,
   -1.093315110e-11,
    6.683939320e+04,
    6.222964380e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.167806520e+00,
    4.752219020e-03,
   -1.837870770e-06,
    3.041902520e-10,
   -1.772327700e-14,
    6.712106500e+04,
    6.635894750e+00,
  },
}
db['C2H'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C2H'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C2H2'] = {}
db['C2H2'].atomicConstituents = { H=2, C=2, }
db['C2H2'].charge = 0
db['C2H2'].M = 2.60372800e-02
db['C2H2'].sigma = 4.10000000
db['C2H2'].epsilon = 209.00000000
db['C2H2'].Lewis = 1.15200000
db['C2H2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    8.086810940e-01,
    2.336156290e-02,
   -3.551718150e-05,
    2.801524370e-08,
   -8.500729740e-12,
    2.642898070e+04,
    1.393970510e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.147569640e+00,
    5.961666640e-03,
   -2.372948520e-06,
    4.674121710e-10,
   -3.612352130e-14,
    2.593599920e+04,
   -1.230281210e+00,
  },
}
db['C2H2'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  5.4922881e-01,
      B = -1.7078109e+02,
      C =  7.2130467e+03,
      D =  1.9955795e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.5338952e-01,
      B =  5.0419792e+01,
      C = -5.6910493e+04,
      D =  1.1190694e+00,
   },
}
db['C2H2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  7.2408606e-01,
      B = -2.7145126e+02,
      C =  1.1112107e+04,
      D =  2.1630756e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.5646287e-01,
      B = -4.3191905e+02,
      C =  2.4326887e+04,
      D =  2.7779508e+00,
   },
}
db['H2CC'] = {}
db['H2CC'].atomicConstituents = { H=2, C=2, }
db['H2CC'].charge = 0
db['H2CC'].M = 2.60372800e-02
db['H2CC'].sigma = 4.10000000
db['H2CC'].epsilon = 209.00000000
db['H2CC'].Lewis = 1.15200000
db['H2CC'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.281548300e+00,
    6.976479100e-03,
   -2.385524400e-06,
   -1.210443200e-09,
    9.818954500e-13,
    4.862179400e+04,
    5.920391000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.278034000e+00,
    4.756280400e-03,
   -1.630100900e-06,
    2.546280600e-10,
   -1.488637900e-14,
    4.831668800e+04,
    6.402370100e-01,
  },
}
db['H2CC'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['H2CC'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C2H3'] = {}
db['C2H3'].atomicConstituents = { H=3, C=2, }
db['C2H3'].charge = 0
db['C2H3'].M = 2.70452200e-02
db['C2H3'].sigma = 4.10000000
db['C2H3'].epsilon = 209.00000000
db['C2H3'].Lewis = 1.15200000
db['C2H3'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.212466450e+00,
    1.514791620e-03,
    2.592094120e-05,
   -3.576578470e-08,
    1.471508730e-11,
    3.485984680e+04,
    8.510540250e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    3.016724000e+00,
    1.033022920e-02,
   -4.680823490e-06,
    1.017632880e-09,
   -8.626070410e-14,
    3.461287390e+04,
    7.787323780e+00,
  },
}
db['C2H3'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C2H3'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C2H4'] = {}
db['C2H4'].atomicConstituents = { H=4, C=2, }
db['C2H4'].charge = 0
db['C2H4'].M = 2.80531600e-02
db['C2H4'].sigma = 3.97100000
db['C2H4'].epsilon = 280.80000000
db['C2H4'].Lewis = 1.40200000
db['C2H4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.959201480e+00,
   -7.570522470e-03,
    5.709902920e-05,
   -6.915887530e-08,
    2.698843730e-11,
    5.089775930e+03,
    4.097330960e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.036111160e+00,
    1.464541510e-02,
   -6.710779150e-06,
    1.472229230e-09,
   -1.257060610e-13,
    4.939886140e+03,
    1.030536930e+01,
  },
}
db['C2H4'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  5.5243600e-01,
      B = -1.6260917e+02,
      C =  6.4734038e+03,
      D =  1.9463233e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.5385054e-01,
      B =  5.1157317e+01,
      C = -5.4731184e+04,
      D =  1.0933538e+00,
   },
}
db['C2H4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  7.7957663e-01,
      B = -4.7857623e+02,
      C =  3.2147858e+04,
      D =  2.1827872e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  4.8277394e-01,
      B = -9.1773465e+02,
      C =  1.1528060e+05,
      D =  4.5824405e+00,
   },
}
db['C2H5'] = {}
db['C2H5'].atomicConstituents = { H=5, C=2, }
db['C2H5'].charge = 0
db['C2H5'].M = 2.90611000e-02
db['C2H5'].sigma = 4.30200000
db['C2H5'].epsilon = 252.30000000
db['C2H5'].Lewis = 1.55100000
db['C2H5'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.306465680e+00,
   -4.186588920e-03,
    4.971428070e-05,
   -5.991266060e-08,
    2.305090040e-11,
    1.284162650e+04,
    4.707209240e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.954656420e+00,
    1.739727220e-02,
   -7.982066680e-06,
    1.752176890e-09,
   -1.496415760e-13,
    1.285752000e+04,
    1.346243430e+01,
  },
}
db['C2H5'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C2H5'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C2H6'] = {}
db['C2H6'].atomicConstituents = { H=6, C=2, }
db['C2H6'].charge = 0
db['C2H6'].M = 3.00690400e-02
db['C2H6'].sigma = 4.30200000
db['C2H6'].epsilon = 252.30000000
db['C2H6'].Lewis = 1.54600000
db['C2H6'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.291424920e+00,
   -5.501542700e-03,
    5.994382880e-05,
   -7.084662850e-08,
    2.686857710e-11,
   -1.152220550e+04,
    2.666823160e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.071881500e+00,
    2.168526770e-02,
   -1.002560670e-05,
    2.214120010e-09,
   -1.900028900e-13,
   -1.142639320e+04,
    1.511561070e+01,
  },
}
db['C2H6'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  5.5619461e-01,
      B = -1.5265690e+02,
      C =  5.6050805e+03,
      D =  1.8241467e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.5422199e-01,
      B =  5.1041684e+01,
      C = -5.1534435e+04,
      D =  1.0006480e+00,
   },
}
db['C2H6'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  8.7089937e-01,
      B = -4.5633731e+02,
      C =  3.1766620e+04,
      D =  1.6351124e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  4.7062424e-01,
      B = -9.6911156e+02,
      C =  1.0907459e+05,
      D =  4.8272647e+00,
   },
}
db['HCCO'] = {}
db['HCCO'].atomicConstituents = { H=1, O=1, C=2, }
db['HCCO'].charge = 0
db['HCCO'].M = 4.10287400e-02
db['HCCO'].sigma = 2.50000000
db['HCCO'].epsilon = 150.00000000
db['HCCO'].Lewis = 1.15200000
db['HCCO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 4000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.251721400e+00,
    1.765502100e-02,
   -2.372910100e-05,
    1.727575900e-08,
   -5.066481100e-12,
    2.005944900e+04,
    1.249041700e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.628205800e+00,
    4.085340100e-03,
   -1.593454700e-06,
    2.862605200e-10,
   -1.940783200e-14,
    1.932721500e+04,
   -3.930259500e+00,
  },
}
db['HCCO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['HCCO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH2CO'] = {}
db['CH2CO'].atomicConstituents = { H=2, O=1, C=2, }
db['CH2CO'].charge = 0
db['CH2CO'].M = 4.20366800e-02
db['CH2CO'].sigma = 3.97000000
db['CH2CO'].epsilon = 436.00000000
db['CH2CO'].Lewis = 1.15200000
db['CH2CO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 3500.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.135836300e+00,
    1.811887210e-02,
   -1.739474740e-05,
    9.343975680e-09,
   -2.014576150e-12,
   -7.042918040e+03,
    1.221564800e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.511297320e+00,
    9.003597450e-03,
   -4.169396350e-06,
    9.233458820e-10,
   -7.948382010e-14,
   -7.551053110e+03,
    6.322472050e-01,
  },
}
db['CH2CO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH2CO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['HCCOH'] = {}
db['HCCOH'].atomicConstituents = { H=2, O=1, C=2, }
db['HCCOH'].charge = 0
db['HCCOH'].M = 4.20366800e-02
db['HCCOH'].sigma = 3.97000000
db['HCCOH'].epsilon = 436.00000000
db['HCCOH'].Lewis = 1.15200000
db['HCCOH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.242373300e+00,
    3.107220100e-02,
   -5.086686400e-05,
    4.313713100e-08,
   -1.401459400e-11,
    8.031614300e+03,
    1.387431900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.923829100e+00,
    6.792360000e-03,
   -2.565856400e-06,
    4.498784100e-10,
   -2.994010100e-14,
    7.264626000e+03,
   -7.601774200e+00,
  },
}
db['HCCOH'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['HCCOH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C2O'] = {}
db['C2O'].atomicConstituents = { H=0, O=1, C=2, }
db['C2O'].charge = 0
db['C2O'].M = 4.00210000e-02
db['C2O'].sigma = 3.82800000
db['C2O'].epsilon = 232.40000000
db['C2O'].Lewis = 1.15200000
db['C2O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.368851000e+00,
    8.241803000e-03,
   -8.765145000e-06,
    5.569262000e-09,
   -1.540009000e-12,
    3.317081000e+04,
    6.713314000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.849809000e+00,
    2.947585000e-03,
   -1.090729000e-06,
    1.792562000e-10,
   -1.115758000e-14,
    3.282055000e+04,
   -6.453226000e-01,
  },
}
db['C2O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C2O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH2CHO'] = {}
db['CH2CHO'].atomicConstituents = { H=3, O=1, C=2, }
db['CH2CHO'].charge = 0
db['CH2CHO'].M = 4.30446200e-02
db['CH2CHO'].sigma = 3.97000000
db['CH2CHO'].epsilon = 436.00000000
db['CH2CHO'].Lewis = 1.15200000
db['CH2CHO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.409062000e+00,
    1.073857400e-02,
    1.891492000e-06,
   -7.158583000e-09,
    2.867385000e-12,
    1.521476600e+03,
    9.558290000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.975670000e+00,
    8.130591000e-03,
   -2.743624000e-06,
    4.070304000e-10,
   -2.176017000e-14,
    4.903218000e+02,
   -5.045251000e+00,
  },
}
db['CH2CHO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH2CHO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH3CHO'] = {}
db['CH3CHO'].atomicConstituents = { H=4, O=1, C=2, }
db['CH3CHO'].charge = 0
db['CH3CHO'].M = 4.40525600e-02
db['CH3CHO'].sigma = 3.97000000
db['CH3CHO'].epsilon = 436.00000000
db['CH3CHO'].Lewis = 1.15200000
db['CH3CHO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.729459500e+00,
   -3.193285800e-03,
    4.753492100e-05,
   -5.745861100e-08,
    2.193111200e-11,
   -2.157287800e+04,
    4.103015900e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.404110800e+00,
    1.172305900e-02,
   -4.226313700e-06,
    6.837245100e-10,
   -4.098486300e-14,
   -2.259312200e+04,
   -3.480791700e+00,
  },
}
db['CH3CHO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH3CHO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH3CO'] = {}
db['CH3CO'].atomicConstituents = { H=3, O=1, C=2, }
db['CH3CO'].charge = 0
db['CH3CO'].M = 4.30440000e-02
db['CH3CO'].sigma = 3.97000000
db['CH3CO'].epsilon = 436.00000000
db['CH3CO'].Lewis = 1.15200000
db['CH3CO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.163425700e+00,
   -2.326161000e-04,
    3.426782000e-05,
   -4.410522700e-08,
    1.727561200e-11,
   -2.657452900e+03,
    7.346828000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.944773100e+00,
    7.866720500e-03,
   -2.886588200e-06,
    4.727087500e-10,
   -2.859986100e-14,
   -3.787307500e+03,
   -5.013675100e+00,
  },
}
db['CH3CO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH3CO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C3H2'] = {}
db['C3H2'].atomicConstituents = { H=2, O=0, C=3, }
db['C3H2'].charge = 0
db['C3H2'].M = 3.80480000e-02
db['C3H2'].sigma = 4.10000000
db['C3H2'].epsilon = 209.00000000
db['C3H2'].Lewis = 1.15200000
db['C3H2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.691077000e+00,
    1.480366000e-02,
   -3.250551000e-06,
   -8.644363000e-09,
    5.284878000e-12,
    5.219072000e+04,
    8.757391000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.530853000e+00,
    5.870316000e-03,
   -1.720777000e-06,
    2.127498000e-10,
   -8.291910000e-15,
    5.115214000e+04,
   -1.122728000e+01,
  },
}
db['C3H2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C3H2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C3H3'] = {}
db['C3H3'].atomicConstituents = { H=3, O=0, C=3, }
db['C3H3'].charge = 0
db['C3H3'].M = 3.90560000e-02
db['C3H3'].sigma = 4.76000000
db['C3H3'].epsilon = 252.00000000
db['C3H3'].Lewis = 1.15200000
db['C3H3'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.351109270e+00,
    3.274112230e-02,
   -4.738271350e-05,
    3.763098080e-08,
   -1.185409230e-11,
    4.010577830e+04,
    1.520589240e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    7.142218800e+00,
    7.619020050e-03,
   -2.674599500e-06,
    4.249148010e-10,
   -2.514754150e-14,
    3.890874270e+04,
   -1.258484360e+01,
  },
}
db['C3H3'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C3H3'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['pC3H4'] = {}
db['pC3H4'].atomicConstituents = { H=4, O=0, C=3, }
db['pC3H4'].charge = 0
db['pC3H4'].M = 4.00640000e-02
db['pC3H4'].sigma = 4.76000000
db['pC3H4'].epsilon = 252.00000000
db['pC3H4'].Lewis = 1.15200000
db['pC3H4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.680386900e+00,
    1.579965100e-02,
    2.507059600e-06,
   -1.365762300e-08,
    6.615428500e-12,
    2.080237400e+04,
    9.876935100e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.025240000e+00,
    1.133654200e-02,
   -4.022339100e-06,
    6.437606300e-10,
   -3.829963500e-14,
    1.962094200e+04,
   -8.604378500e+00,
  },
}
db['pC3H4'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['pC3H4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['aC3H4'] = {}
db['aC3H4'].atomicConstituents = { H=4, O=0, C=3, }
db['aC3H4'].charge = 0
db['aC3H4'].M = 4.00640000e-02
db['aC3H4'].sigma = 4.76000000
db['aC3H4'].epsilon = 252.00000000
db['aC3H4'].Lewis = 1.15200000
db['aC3H4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.613044500e+00,
    1.212257500e-02,
    1.853988000e-05,
   -3.452514900e-08,
    1.533507900e-11,
    2.154156700e+04,
    1.022613900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.316872200e+00,
    1.113372800e-02,
   -3.962937800e-06,
    6.356423800e-10,
   -3.787554000e-14,
    2.011749500e+04,
   -1.099576600e+01,
  },
}
db['aC3H4'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['aC3H4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['cC3H4'] = {}
db['cC3H4'].atomicConstituents = { H=4, O=0, C=3, }
db['cC3H4'].charge = 0
db['cC3H4'].M = 4.00640000e-02
db['cC3H4'].sigma = 4.76000000
db['cC3H4'].epsilon = 252.00000000
db['cC3H4'].Lewis = 1.15200000
db['cC3H4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -2.462104700e-02,
    2.319721500e-02,
   -1.847435700e-06,
   -1.592759300e-08,
    8.684615500e-12,
    3.233413700e+04,
    2.272976200e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.699993100e+00,
    1.035737200e-02,
   -3.455116700e-06,
    5.065294900e-10,
   -2.668227600e-14,
    3.019905100e+04,
   -1.337877000e+01,
  },
}
db['cC3H4'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['cC3H4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['aC3H5'] = {}
db['aC3H5'].atomicConstituents = { H=5, C=3, }
db['aC3H5'].charge = 0
db['aC3H5'].M = 4.10718000e-02
db['aC3H5'].sigma = 4.98200000
db['aC3H5'].epsilon = 266.80000000
db['aC3H5'].Lewis = 1.15200000
db['aC3H5'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.363183500e+00,
    1.981382100e-02,
    1.249706000e-05,
   -3.335555500e-08,
    1.584657100e-11,
    1.924562900e+04,
    1.717321400e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.500787700e+00,
    1.432473100e-02,
   -5.678163200e-06,
    1.108080100e-09,
   -9.036388700e-14,
    1.748244900e+04,
   -1.124305000e+01,
  },
}
db['aC3H5'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['aC3H5'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH3CCH2'] = {}
db['CH3CCH2'].atomicConstituents = { H=5, O=0, C=3, }
db['CH3CCH2'].charge = 0
db['CH3CCH2'].M = 4.10720000e-02
db['CH3CCH2'].sigma = 4.98200000
db['CH3CCH2'].epsilon = 266.80000000
db['CH3CCH2'].Lewis = 1.15200000
db['CH3CCH2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.732920900e+00,
    2.239462000e-02,
   -5.149061100e-06,
   -6.759646600e-09,
    3.825321100e-12,
    2.904049800e+04,
    1.656887800e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.425552800e+00,
    1.551107200e-02,
   -5.667835000e-06,
    7.922438800e-10,
   -1.687803400e-14,
    2.784302700e+04,
   -3.352718400e+00,
  },
}
db['CH3CCH2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH3CCH2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['CH3CHCH'] = {}
db['CH3CHCH'].atomicConstituents = { H=5, O=0, C=3, }
db['CH3CHCH'].charge = 0
db['CH3CHCH'].M = 4.10720000e-02
db['CH3CHCH'].sigma = 4.98200000
db['CH3CHCH'].epsilon = 266.80000000
db['CH3CHCH'].Lewis = 1.15200000
db['CH3CHCH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    9.137293100e-01,
    2.643234300e-02,
   -1.175895000e-05,
   -2.303567800e-09,
    2.771548800e-12,
    3.091686700e+04,
    1.998926900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.372528100e+00,
    1.578050900e-02,
   -5.992285000e-06,
    9.308966400e-10,
   -3.655096600e-14,
    2.961476000e+04,
   -3.418647800e+00,
  },
}
db['CH3CHCH'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['CH3CHCH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C3H6'] = {}
db['C3H6'].atomicConstituents = { H=6, C=3, }
db['C3H6'].charge = 0
db['C3H6'].M = 4.20797400e-02
db['C3H6'].sigma = 4.98200000
db['C3H6'].epsilon = 266.80000000
db['C3H6'].Lewis = 1.15200000
db['C3H6'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.493307000e+00,
    2.092518000e-02,
    4.486794000e-06,
   -1.668912000e-08,
    7.158146000e-12,
    1.074826000e+03,
    1.614534000e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.732257000e+00,
    1.490834000e-02,
   -4.949899000e-06,
    7.212022000e-10,
   -3.766204000e-14,
   -9.235703000e+02,
   -1.331335000e+01,
  },
}
db['C3H6'].viscosity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  5.2642893e-01,
      B = -2.4304494e+02,
      C =  1.4490001e+04,
      D =  2.1036650e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.4243372e-01,
      B =  8.3055174e+00,
      C = -6.1290810e+04,
      D =  1.1264132e+00,
   },
}
db['C3H6'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 2,
   segment0 = {
      T_lower = 300.0,
      T_upper = 1000.0,
      A =  7.5434495e-01,
      B = -5.6817108e+02,
      C =  3.9706666e+04,
      D =  2.3579094e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  4.6796950e-01,
      B = -9.8032164e+02,
      C =  1.2025017e+05,
      D =  4.6607118e+00,
   },
}
db['C2H3CHO'] = {}
db['C2H3CHO'].atomicConstituents = { H=4, O=1, C=3, }
db['C2H3CHO'].charge = 0
db['C2H3CHO'].M = 5.60630000e-02
db['C2H3CHO'].sigma = 5.17600000
db['C2H3CHO'].epsilon = 357.00000000
db['C2H3CHO'].Lewis = 1.15200000
db['C2H3CHO'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 298.15, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.152958400e+00,
    2.804021400e-02,
   -1.507215300e-05,
    1.590584200e-09,
    8.493037100e-13,
   -1.041769400e+04,
    2.145327900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.835318000e+00,
    1.977260100e-02,
   -1.042662800e-05,
    2.652580300e-09,
   -2.627820700e-13,
   -1.155783700e+04,
    1.885314400e+00,
  },
}
db['C2H3CHO'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C2H3CHO'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['nC3H7'] = {}
db['nC3H7'].atomicConstituents = { H=7, C=3, }
db['nC3H7'].charge = 0
db['nC3H7'].M = 4.30876800e-02
db['nC3H7'].sigma = 4.98200000
db['nC3H7'].epsilon = 266.80000000
db['nC3H7'].Lewis = 1.15200000
db['nC3H7'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.049117300e+00,
    2.600897300e-02,
    2.354251600e-06,
   -1.959513200e-08,
    9.372020700e-12,
    1.031234600e+04,
    2.113603400e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    7.709747900e+00,
    1.603148500e-02,
   -5.272023800e-06,
    7.588835200e-10,
   -3.886271900e-14,
    7.976223600e+03,
   -1.551529700e+01,
  },
}
db['nC3H7'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['nC3H7'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['iC3H7'] = {}
db['iC3H7'].atomicConstituents = { H=7, O=0, C=3, }
db['iC3H7'].charge = 0
db['iC3H7'].M = 4.30870000e-02
db['iC3H7'].sigma = 4.98200000
db['iC3H7'].epsilon = 266.80000000
db['iC3H7'].Lewis = 1.15200000
db['iC3H7'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.444919900e+00,
    2.099911200e-02,
    7.703622200e-06,
   -1.847625300e-08,
    7.128296200e-12,
    9.422372400e+03,
    2.011631700e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.519274100e+00,
    1.722010400e-02,
   -5.736421700e-06,
    8.413073200e-10,
   -4.456591300e-14,
    7.322719300e+03,
   -9.083021500e+00,
  },
}
db['iC3H7'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['iC3H7'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C3H8'] = {}
db['C3H8'].atomicConstituents = { H=8, C=3, }
db['C3H8'].charge = 0
db['C3H8'].M = 4.40956200e-02
db['C3H8'].sigma = 4.98200000
db['C3H8'].epsilon = 266.80000000
db['C3H8'].Lewis = 1.15200000
db['C3H8'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    9.335538100e-01,
    2.642457900e-02,
    6.105972700e-06,
   -2.197749900e-08,
    9.514925300e-12,
   -1.395852000e+04,
    1.920169100e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    7.534136800e+00,
    1.887223900e-02,
   -6.271849100e-06,
    9.147564900e-10,
   -4.783806900e-14,
   -1.646751600e+04,
   -1.789234900e+01,
  },
}
db['C3H8'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C3H8'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C4H'] = {}
db['C4H'].atomicConstituents = { H=1, O=0, C=4, }
db['C4H'].charge = 0
db['C4H'].M = 4.90510000e-02
db['C4H'].sigma = 5.18000000
db['C4H'].epsilon = 357.00000000
db['C4H'].Lewis = 1.15200000
db['C4H'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.318629500e+00,
    3.858295600e-02,
   -7.138562300e-05,
    6.535635900e-08,
   -2.261766600e-11,
    9.545610600e+04,
    1.556758300e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    7.769759300e+00,
    4.982997600e-03,
   -1.762854600e-06,
    2.814428400e-10,
   -1.668986900e-14,
    9.434590000e+04,
   -1.416527400e+01,
  },
}
db['C4H'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C4H'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C4H2'] = {}
db['C4H2'].atomicConstituents = { H=2, O=0, C=4, }
db['C4H2'].charge = 0
db['C4H2'].M = 5.00590000e-02
db['C4H2'].sigma = 5.18000000
db['C4H2'].epsilon = 357.00000000
db['C4H2'].Lewis = 1.15200000
db['C4H2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -3.920103000e-01,
    5.193756500e-02,
   -9.173734000e-05,
    8.047198600e-08,
   -2.689821800e-11,
    5.484526600e+04,
    2.095779400e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    8.663770800e+00,
    6.724718900e-03,
   -2.359339700e-06,
    3.750638000e-10,
   -2.223094000e-14,
    5.325227500e+04,
   -2.109350300e+01,
  },
}
db['C4H2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C4H2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['H2C4O'] = {}
db['H2C4O'].atomicConstituents = { H=2, O=1, C=4, }
db['H2C4O'].charge = 0
db['H2C4O'].M = 6.60580000e-02
db['H2C4O'].sigma = 5.18000000
db['H2C4O'].epsilon = 357.00000000
db['H2C4O'].Lewis = 1.15200000
db['H2C4O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 4000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    4.810971000e+00,
    1.313999000e-02,
    9.865073000e-07,
   -6.120720000e-09,
    1.640003000e-12,
    2.545803000e+04,
    2.113424000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.026888000e+01,
    4.896164000e-03,
   -4.885081000e-07,
   -2.708566000e-10,
    5.107013000e-14,
    2.346903000e+04,
   -2.815985000e+01,
  },
}
db['H2C4O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['H2C4O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['n-C4H3'] = {}
db['n-C4H3'].atomicConstituents = { H=3, O=0, C=4, }
db['n-C4H3'].charge = 0
db['n-C4H3'].M = 5.10660000e-02
db['n-C4H3'].sigma = 5.18000000
db['n-C4H3'].epsilon = 357.00000000
db['n-C4H3'].Lewis = 1.15200000
db['n-C4H3'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -3.168411300e-01,
    4.691210000e-02,
   -6.809381000e-05,
    5.317992100e-08,
   -1.652300500e-11,
    6.247619900e+04,
    2.462255900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.432827900e+00,
    1.686098100e-02,
   -9.431310900e-06,
    2.570389500e-09,
   -2.745630900e-13,
    6.160068000e+04,
   -1.567398100e+00,
  },
}
db['n-C4H3'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['n-C4H3'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['i-C4H3'] = {}
db['i-C4H3'].atomicConstituents = { H=3, O=0, C=4, }
db['i-C4H3'].charge = 0
db['i-C4H3'].M = 5.10660000e-02
db['i-C4H3'].sigma = 5.18000000
db['i-C4H3'].epsilon = 357.00000000
db['i-C4H3'].Lewis = 1.15200000
db['i-C4H3'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.083041200e+00,
    4.083427400e-02,
   -6.215968500e-05,
    5.167935800e-08,
   -1.702918400e-11,
    5.800512900e+04,
    1.361746200e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    9.097816500e+00,
    9.220711900e-03,
   -3.387844100e-06,
    4.916049800e-10,
   -1.452978000e-14,
    5.660057400e+04,
   -1.980259700e+01,
  },
}
db['i-C4H3'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['i-C4H3'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C4H4'] = {}
db['C4H4'].atomicConstituents = { H=4, O=0, C=4, }
db['C4H4'].charge = 0
db['C4H4'].M = 5.20740000e-02
db['C4H4'].sigma = 5.18000000
db['C4H4'].epsilon = 357.00000000
db['C4H4'].Lewis = 1.15200000
db['C4H4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -1.915247900e+00,
    5.275087800e-02,
   -7.165594400e-05,
    5.507242300e-08,
   -1.728622800e-11,
    3.297850400e+04,
    3.141998300e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    6.650709200e+00,
    1.612943400e-02,
   -7.193887500e-06,
    1.498178700e-09,
   -1.186411000e-13,
    3.119599200e+04,
   -9.795211800e+00,
  },
}
db['C4H4'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C4H4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['n-C4H5'] = {}
db['n-C4H5'].atomicConstituents = { H=5, O=0, C=4, }
db['n-C4H5'].charge = 0
db['n-C4H5'].M = 5.30820000e-02
db['n-C4H5'].sigma = 5.18000000
db['n-C4H5'].epsilon = 357.00000000
db['n-C4H5'].Lewis = 1.15200000
db['n-C4H5'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.630532100e-01,
    3.983013700e-02,
   -3.400012800e-05,
    1.514723300e-08,
   -2.466582500e-12,
    4.142976600e+04,
    2.353616300e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    9.850197800e+00,
    1.077900800e-02,
   -1.367212500e-06,
   -7.720053500e-10,
    1.836631400e-13,
    3.884030100e+04,
   -2.600184600e+01,
  },
}
db['n-C4H5'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['n-C4H5'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['i-C4H5'] = {}
db['i-C4H5'].atomicConstituents = { H=5, O=0, C=4, }
db['i-C4H5'].charge = 0
db['i-C4H5'].M = 5.30820000e-02
db['i-C4H5'].sigma = 5.18000000
db['i-C4H5'].epsilon = 357.00000000
db['i-C4H5'].Lewis = 1.15200000
db['i-C4H5'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -1.993290000e-02,
    3.800567200e-02,
   -2.755945000e-05,
    7.783555100e-09,
    4.020938300e-13,
    3.749622300e+04,
    2.439424100e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.022909200e+01,
    9.485013800e-03,
   -9.040644500e-08,
   -1.259610000e-09,
    2.478146800e-13,
    3.464281200e+04,
   -2.856452900e+01,
  },
}
db['i-C4H5'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['i-C4H5'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C4H6'] = {}
db['C4H6'].atomicConstituents = { H=6, O=0, C=4, }
db['C4H6'].charge = 0
db['C4H6'].M = 5.40900000e-02
db['C4H6'].sigma = 5.18000000
db['C4H6'].epsilon = 357.00000000
db['C4H6'].Lewis = 1.15200000
db['C4H6'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.128446500e-01,
    3.436902200e-02,
   -1.110739200e-05,
   -9.210666000e-09,
    6.206517900e-12,
    1.180227000e+04,
    2.308999600e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    8.867313400e+00,
    1.491867000e-02,
   -3.154871600e-06,
   -4.184133000e-10,
    1.576125800e-13,
    9.133851600e+03,
   -2.332817100e+01,
  },
}
db['C4H6'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C4H6'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C4H612'] = {}
db['C4H612'].atomicConstituents = { H=6, O=0, C=4, }
db['C4H612'].charge = 0
db['C4H612'].M = 5.40900000e-02
db['C4H612'].sigma = 5.18000000
db['C4H612'].epsilon = 357.00000000
db['C4H612'].Lewis = 1.15200000
db['C4H612'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.023467000e+00,
    3.495919000e-02,
   -2.200905000e-05,
    6.942272000e-09,
   -7.879187000e-13,
    1.811799000e+04,
    1.975066000e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.781557000e+01,
   -4.257502000e-03,
    1.051185000e-05,
   -4.473844000e-09,
    5.848138000e-13,
    1.267342000e+04,
   -6.982662000e+01,
  },
}
db['C4H612'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C4H612'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C4H7'] = {}
db['C4H7'].atomicConstituents = { H=7, O=0, C=4, }
db['C4H7'].charge = 0
db['C4H7'].M = 5.50980000e-02
db['C4H7'].sigma = 5.17600000
db['C4H7'].epsilon = 357.00000000
db['C4H7'].Lewis = 1.15200000
db['C4H7'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.869825400e-01,
    3.696449500e-02,
   -8.627744100e-06,
   -1.505182100e-08,
    8.989126300e-12,
    2.055130100e+04,
    2.448446700e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.196339200e+01,
    1.142530500e-02,
    7.894890900e-07,
   -1.985887200e-09,
    3.687364500e-13,
    1.696297700e+04,
   -3.754290800e+01,
  },
}
db['C4H7'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C4H7'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C4H81'] = {}
db['C4H81'].atomicConstituents = { H=8, O=0, C=4, }
db['C4H81'].charge = 0
db['C4H81'].M = 5.61060000e-02
db['C4H81'].sigma = 5.17600000
db['C4H81'].epsilon = 357.00000000
db['C4H81'].Lewis = 1.15200000
db['C4H81'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.181138000e+00,
    3.085338000e-02,
    5.086524700e-06,
   -2.465488800e-08,
    1.111019300e-11,
   -1.790400400e+03,
    2.106246900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.053584100e+00,
    3.435050700e-02,
   -1.588319700e-05,
    3.308966200e-09,
   -2.536104500e-13,
   -2.139723100e+03,
    1.554320100e+01,
  },
}
db['C4H81'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C4H81'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C6H2'] = {}
db['C6H2'].atomicConstituents = { H=2, O=0, C=6, }
db['C6H2'].charge = 0
db['C6H2'].M = 7.40800000e-02
db['C6H2'].sigma = 5.18000000
db['C6H2'].epsilon = 357.00000000
db['C6H2'].Lewis = 1.15200000
db['C6H2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -1.593262400e+00,
    8.053014500e-02,
   -1.480064900e-04,
    1.330003100e-07,
   -4.533231300e-11,
    8.327322700e+04,
    2.798087300e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.322628100e+01,
    7.390430200e-03,
   -2.271538100e-06,
    2.587521700e-10,
   -5.535674100e-15,
    8.056525800e+04,
   -4.120117600e+01,
  },
}
db['C6H2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C6H2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C6H3'] = {}
db['C6H3'].atomicConstituents = { H=3, O=0, C=6, }
db['C6H3'].charge = 0
db['C6H3'].M = 7.50880000e-02
db['C6H3'].sigma = 5.18000000
db['C6H3'].epsilon = 357.00000000
db['C6H3'].Lewis = 1.15200000
db['C6H3'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    1.179061900e+00,
    5.554736000e-02,
   -7.307616800e-05,
    5.207673600e-08,
   -1.504696400e-11,
    8.564731200e+04,
    1.917919900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    5.818834300e+00,
    2.793340800e-02,
   -1.782542700e-05,
    5.370253600e-09,
   -6.170762700e-13,
    8.518825000e+04,
   -9.214782700e-01,
  },
}
db['C6H3'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C6H3'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['l-C6H4'] = {}
db['l-C6H4'].atomicConstituents = { H=4, O=0, C=6, }
db['l-C6H4'].charge = 0
db['l-C6H4'].M = 7.60960000e-02
db['l-C6H4'].sigma = 5.34900000
db['l-C6H4'].epsilon = 412.30000000
db['l-C6H4'].Lewis = 1.15200000
db['l-C6H4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.959022500e-01,
    5.805331800e-02,
   -6.776675600e-05,
    4.337676200e-08,
   -1.141886400e-11,
    6.000137100e+04,
    2.231897000e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.271518200e+01,
    1.383966200e-02,
   -4.376544000e-06,
    3.154163600e-10,
    4.661902600e-14,
    5.703114800e+04,
   -3.946460000e+01,
  },
}
db['l-C6H4'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['l-C6H4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['c-C6H4'] = {}
db['c-C6H4'].atomicConstituents = { H=4, O=0, C=6, }
db['c-C6H4'].charge = 0
db['c-C6H4'].M = 7.60960000e-02
db['c-C6H4'].sigma = 5.29000000
db['c-C6H4'].epsilon = 464.80000000
db['c-C6H4'].Lewis = 1.15200000
db['c-C6H4'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -3.099126800e+00,
    5.403056400e-02,
   -4.083900400e-05,
    1.073883700e-08,
    9.807849000e-13,
    5.220571100e+04,
    3.741520700e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.384920900e+01,
    7.880792000e-03,
    1.824383600e-06,
   -2.116916600e-09,
    3.745997700e-13,
    4.744634000e+04,
   -5.040495300e+01,
  },
}
db['c-C6H4'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['c-C6H4'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['A1'] = {}
db['A1'].atomicConstituents = { H=6, O=0, C=6, }
db['A1'].charge = 0
db['A1'].M = 7.81120000e-02
db['A1'].sigma = 5.29000000
db['A1'].epsilon = 464.80000000
db['A1'].Lewis = 1.15200000
db['A1'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -4.899868000e+00,
    5.980693200e-02,
   -3.671008700e-05,
    3.274039900e-09,
    3.760088600e-12,
    9.182457000e+03,
    4.409564200e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.724699400e+01,
    3.842016400e-03,
    8.277623200e-06,
   -4.896112000e-09,
    7.606454500e-13,
    2.664605500e+03,
   -7.194517500e+01,
  },
}
db['A1'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['A1'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['A1-'] = {}
db['A1-'].atomicConstituents = { H=5, O=0, C=6, }
db['A1-'].charge = 0
db['A1-'].M = 7.71040000e-02
db['A1-'].sigma = 5.29000000
db['A1-'].epsilon = 464.80000000
db['A1-'].Lewis = 1.15200000
db['A1-'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -4.907614700e+00,
    5.979077100e-02,
   -4.563982700e-05,
    1.496499300e-08,
   -9.176782600e-13,
    3.873341000e+04,
    4.656778000e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.449343900e+01,
    7.571268800e-03,
    3.789454200e-06,
   -3.076950000e-09,
    5.134782000e-13,
    3.318997700e+04,
   -5.428894000e+01,
  },
}
db['A1-'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['A1-'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C6H5O'] = {}
db['C6H5O'].atomicConstituents = { H=5, O=1, C=6, }
db['C6H5O'].charge = 0
db['C6H5O'].M = 9.31030000e-02
db['C6H5O'].sigma = 5.29000000
db['C6H5O'].epsilon = 464.80000000
db['C6H5O'].Lewis = 1.15200000
db['C6H5O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -1.821943300e+00,
    4.812251000e-02,
   -4.679230200e-06,
   -3.401859400e-08,
    1.864963700e-11,
    4.242918000e+03,
    3.352619900e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.383398400e+01,
    1.761840300e-02,
   -6.069625700e-06,
    9.198817300e-10,
   -5.044918100e-14,
   -6.921254900e+02,
   -5.039299000e+01,
  },
}
db['C6H5O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C6H5O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C6H5OH'] = {}
db['C6H5OH'].atomicConstituents = { H=6, O=1, C=6, }
db['C6H5OH'].charge = 0
db['C6H5OH'].M = 9.41110000e-02
db['C6H5OH'].sigma = 5.29000000
db['C6H5OH'].epsilon = 464.80000000
db['C6H5OH'].Lewis = 1.15200000
db['C6H5OH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -1.695653900e+00,
    5.227129900e-02,
   -7.202405000e-06,
   -3.585960300e-08,
    2.044907300e-11,
   -1.328412100e+04,
    3.254216000e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.491207300e+01,
    1.837813500e-02,
   -6.198312800e-06,
    9.198322100e-10,
   -4.920956500e-14,
   -1.837519900e+04,
   -5.592410300e+01,
  },
}
db['C6H5OH'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C6H5OH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C5H6'] = {}
db['C5H6'].atomicConstituents = { H=6, O=0, C=5, }
db['C5H6'].charge = 0
db['C5H6'].M = 6.61010000e-02
db['C5H6'].sigma = 5.18000000
db['C5H6'].epsilon = 357.00000000
db['C5H6'].Lewis = 1.15200000
db['C5H6'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 298.15, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -2.897895800e+00,
    4.348477700e-02,
   -3.351100500e-06,
   -3.110375600e-08,
    1.691244400e-11,
    1.508474200e+04,
    3.689476000e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.062432000e+01,
    1.773544800e-02,
   -6.233044600e-06,
    9.730831700e-10,
   -5.550013000e-14,
    1.077218800e+04,
   -3.577342200e+01,
  },
}
db['C5H6'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C5H6'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C5H5'] = {}
db['C5H5'].atomicConstituents = { H=5, O=0, C=5, }
db['C5H5'].charge = 0
db['C5H5'].M = 6.50930000e-02
db['C5H5'].sigma = 5.18000000
db['C5H5'].epsilon = 357.00000000
db['C5H5'].Lewis = 1.15200000
db['C5H5'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -9.590371800e-01,
    3.139685900e-02,
    2.672379400e-05,
   -6.894187200e-08,
    3.330185600e-11,
    3.072912000e+04,
    2.907281600e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.084406600e+01,
    1.539283700e-02,
   -5.563042100e-06,
    9.018937100e-10,
   -5.415653100e-14,
    2.690056600e+04,
   -3.525494800e+01,
  },
}
db['C5H5'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C5H5'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C5H4O'] = {}
db['C5H4O'].atomicConstituents = { H=4, O=1, C=5, }
db['C5H4O'].charge = 0
db['C5H4O'].M = 8.00840000e-02
db['C5H4O'].sigma = 5.29000000
db['C5H4O'].epsilon = 464.80000000
db['C5H4O'].Lewis = 1.15200000
db['C5H4O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 3000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -2.391535500e+00,
    4.736368000e-02,
   -3.072817100e-05,
    7.803155200e-09,
   -2.514572900e-13,
    4.374015200e+03,
    3.459433700e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    4.792724200e+00,
    2.922168000e-02,
   -1.599748600e-05,
    4.206904900e-09,
   -4.281517900e-13,
    2.284928600e+03,
   -3.013189300e+00,
  },
}
db['C5H4O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C5H4O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C5H4OH'] = {}
db['C5H4OH'].atomicConstituents = { H=5, O=1, C=5, }
db['C5H4OH'].charge = 0
db['C5H4OH'].M = 8.10920000e-02
db['C5H4OH'].sigma = 5.29000000
db['C5H4OH'].epsilon = 464.80000000
db['C5H4OH'].Lewis = 1.15200000
db['C5H4OH'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
   -1.282223600e+00,
    4.904116000e-02,
   -1.368899700e-05,
   -2.913385800e-08,
    1.900696400e-11,
    8.008709800e+03,
    3.079835800e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.336791200e+01,
    1.520578500e-02,
   -5.459225800e-06,
    8.813486600e-10,
   -5.277445400e-14,
    3.841150600e+03,
   -4.592083900e+01,
  },
}
db['C5H4OH'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C5H4OH'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['C5H5O'] = {}
db['C5H5O'].atomicConstituents = { H=5, O=1, C=5, }
db['C5H5O'].charge = 0
db['C5H5O'].M = 8.10920000e-02
db['C5H5O'].sigma = 5.29000000
db['C5H5O'].epsilon = 464.80000000
db['C5H5O'].Lewis = 1.15200000
db['C5H5O'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 200.00, 1000.00, 6000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.304283500e-01,
    3.232269100e-02,
    2.890044300e-05,
   -7.067997700e-08,
    3.340689100e-11,
    8.075308200e+03,
    2.533097400e+01,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    1.260642200e+01,
    1.674726000e-02,
   -6.109857400e-06,
    9.967655700e-10,
   -6.011320100e-14,
    3.931345500e+03,
   -4.260427700e+01,
  },
}
db['C5H5O'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['C5H5O'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
db['Ar'] = {}
db['Ar'].atomicConstituents = { Ar=1, }
db['Ar'].charge = 0
db['Ar'].M = 3.99480000e-02
db['Ar'].sigma = 3.33000000
db['Ar'].epsilon = 136.50000000
db['Ar'].Lewis = 1.17300000
db['Ar'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    2.500000000e+00,
    0.000000000e+00,
    0.000000000e+00,
    0.000000000e+00,
    0.000000000e+00,
   -7.453750000e+02,
    4.366000000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.500000000e+00,
    0.000000000e+00,
    0.000000000e+00,
    0.000000000e+00,
    0.000000000e+00,
   -7.453750000e+02,
    4.366000000e+00,
  },
}
db['Ar'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.1205763e-01,
      B = -6.7714354e+01,
      C =  1.9040660e+02,
      D =  2.1588272e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.9357334e-01,
      B =  7.0953943e+01,
      C = -2.8386007e+04,
      D =  1.4856447e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  7.6608935e-01,
      B =  6.7867215e+02,
      C = -8.4991417e+05,
      D =  7.7935167e-01,
   },
}
db['Ar'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.0968928e-01,
      B = -7.0892249e+01,
      C =  5.8420624e+02,
      D =  1.9337152e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  6.9075463e-01,
      B =  6.2676058e+01,
      C = -2.5667413e+04,
      D =  1.2664189e+00,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  7.6269502e-01,
      B =  6.2341752e+02,
      C = -7.1899552e+05,
      D =  5.6927918e-01,
   },
}
db['N2'] = {}
db['N2'].atomicConstituents = { N=2, }
db['N2'].charge = 0
db['N2'].M = 2.80134000e-02
db['N2'].sigma = 3.62100000
db['N2'].epsilon = 97.53000000
db['N2'].Lewis = 1.15200000
db['N2'].thermoCoeffs = {
  origin = 'GRIMECH',
  nsegments = 2, 
  T_break_points = { 300.00, 1000.00, 5000.00, },
  T_blend_ranges = { 400.0, },
  segment0 = {
    0.000000000e+00,
    0.000000000e+00,
    3.298677000e+00,
    1.408240400e-03,
   -3.963222000e-06,
    5.641515000e-09,
   -2.444854000e-12,
   -1.020899900e+03,
    3.950372000e+00,
  },
  segment1 = {
    0.000000000e+00,
    0.000000000e+00,
    2.926640000e+00,
    1.487976800e-03,
   -5.684760000e-07,
    1.009703800e-10,
   -6.753351000e-15,
   -9.227977000e+02,
    5.980528000e+00,
  },
}
db['N2'].viscosity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  6.2526577e-01,
      B = -3.1779652e+01,
      C = -1.6407983e+03,
      D =  1.7454992e+00,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.7395209e-01,
      B =  5.6152222e+02,
      C = -1.7394809e+05,
      D = -3.9335958e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  8.8503551e-01,
      B =  9.0902171e+02,
      C = -7.3129061e+05,
      D = -5.3503838e-01,
   },
}
db['N2'].thermal_conductivity = {
   model = 'CEA',
   nsegments = 3,
   segment0 = {
      T_lower = 200.0,
      T_upper = 1000.0,
      A =  8.5439436e-01,
      B =  1.0573224e+02,
      C = -1.2347848e+04,
      D =  4.7793128e-01,
   },
   segment1 = {
      T_lower = 1000.0,
      T_upper = 5000.0,
      A =  8.8407146e-01,
      B =  1.3357293e+02,
      C = -1.1429640e+04,
      D =  2.4417019e-01,
   },
   segment2 = {
      T_lower = 5000.0,
      T_upper = 15000.0,
      A =  2.4176185e+00,
      B =  8.0477749e+03,
      C =  3.1055802e+06,
      D = -1.4517761e+01,
   },
}
