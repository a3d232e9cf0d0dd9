-- A fixture mechanism for the rate-constant forms that no mechanism of the reference's examples uses:
-- 'Arrhenius2' (k = exp(logA + B T - C/T), src/kinetics/rate_constant.d:82-121) and the
-- Lindemann-Hinshelwood and Yungster-Rabinowitz fall-off forms (rate_constant.d:123-161, 295-355),
-- next to plain and third-body Arrhenius reactions.  It is processed by the reference's own prep_chem
-- (tests/golden/make_fixtures.sh) with the Jachimowski-1992 species.
--
-- The reactions are the H2-O2 core of examples/kinetics/hydrogen-ignition-delay/Jachimowski-1992.lua
-- and Stanford-2011.lua:
--   * J92 r1, r2 and r11 restated as Arrhenius2.  prep_chem applies no unit conversion to logA, so
--     logA = ln(A [cm^3/mol/s] * 1e-6) is already in SI; r2 carries B = 2e-5 /K so that the B T term
--     is exercised (this changes its rate by a factor exp(B T), 1.02 to 1.06 over 1000-3000 K);
--   * Stanford-2011 r2d (H + O2 (+ M)) without its Troe table, i.e. Lindemann-Hinshelwood;
--   * Stanford-2011 r3 (H2O2 (+ M)) with a Yungster-Rabinowitz table in place of Troe:
--     F_c = a exp(-b/T) + (1 - a) exp(-c/T) with a = 0.735, b = 94 K, c = 1756 K.

Config{
   odeStep = {method='alpha-qss'},
   tightTempCoupling = true,
}

S = 1.0/1.98720

Reaction{
   'H2 + O2 <=> H + HO2',
   fr={'Arrhenius2', logA=18.064005800013632, B=0.0, C=2.86020e04},
   label='r1'
}

Reaction{
   'H + O2 <=> OH + O',
   fr={'Arrhenius2', logA=19.209138104316636, B=2.0e-5, C=8.45974e03},
   label='r2'
}

Reaction{
   'O + H2 <=> OH + H',
   fr={'Arrhenius', A=5.06e4, n=2.67, C=3.16737e03},
   label='r3'
}

Reaction{
   'OH + H2 <=> H2O + H',
   fr={'Arrhenius', A=2.16e08, n=1.51, C=1.72720e03},
   label='r4'
}

Reaction{
   'OH + OH <=> H2O + O',
   fr={'Arrhenius', A=1.5e09, n=1.14, C=0.0},
   label='r5'
}

Reaction{
   'H + OH + M <=> H2O + M',
   fr={'Arrhenius', A=8.62e21, n=-2.0, C=0.0},
   efficiencies={['H2']=2.5,['H2O']=16.0},
   label='r6'
}

Reaction{
   'H + H + M <=> H2 + M',
   fr={'Arrhenius', A=7.3e17, n=-1.0, C=0.0},
   efficiencies={['H2']=2.5,['H2O']=16.0},
   label='r7'
}

Reaction{
   'HO2 + H <=> OH + OH',
   fr={'Arrhenius2', logA=18.826145852060530, B=0.0, C=5.03556e02},
   label='r11'
}

Reaction{
   'HO2 + OH <=> H2O + O2',
   fr={'Arrhenius', A=2.0e13, n=0.0, C=0.0},
   label='r13'
}

Reaction{
   'H + O2 (+ M) <=> HO2 (+ M)',
   fr={'pressure dependent',
       kInf={A=5.59e13, n=0.2, C=0.0},
       k0={A=2.65e19, n=-1.3, C=0.0}
   },
   efficiencies={H2=2.5,H2O2=12.0,H2O=16.0},
   label='lh'
}

Reaction{
   'H2O2 (+ M) <=> 2OH (+ M)',
   fr={'pressure dependent',
       kInf={A=8.59e14, n=0.0, C=48560*S},
       k0={A=9.55e15, n=0.0, C=42203*S},
       YR={a=0.735, b=94.0, c=1756.0}
   },
   efficiencies={N2=1.5,H2=2.5,H2O=15,H2O2=15},
   label='yr'
}
