
mechanism = {}

mechanism[1] = {
  type = 'V-T',
  p = 'N2', q = 'N',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=180.000, b=0.026200}}
}

mechanism[2] = {
  type = 'V-T',
  p = 'N2', q = 'O',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=72.400, b=0.015000}}
}

mechanism[3] = {
  type = 'V-T',
  p = 'N2', q = 'N2',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=221.000, b=0.029000}}
}

mechanism[4] = {
  type = 'V-T',
  p = 'N2', q = 'O2',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=229.000, b=0.029500}}
}

mechanism[5] = {
  type = 'V-T',
  p = 'N2', q = 'NO',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=225.000, b=0.029300}}
}

mechanism[6] = {
  type = 'V-T',
  p = 'O2', q = 'N',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=72.400, b=0.015000}}
}

mechanism[7] = {
  type = 'V-T',
  p = 'O2', q = 'O',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=47.700, b=0.059000}}
}

mechanism[8] = {
  type = 'V-T',
  p = 'O2', q = 'N2',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=134.000, b=0.029500}}
}

mechanism[9] = {
  type = 'V-T',
  p = 'O2', q = 'O2',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=138.000, b=0.030000}}
}

mechanism[10] = {
  type = 'V-T',
  p = 'O2', q = 'NO',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=136.000, b=0.029800}}
}

mechanism[11] = {
  type = 'V-T',
  p = 'NO', q = 'N2',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=49.500, b=0.042000}}
}

mechanism[12] = {
  type = 'V-T',
  p = 'NO', q = 'O2',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=49.500, b=0.042000}}
}

mechanism[13] = {
  type = 'V-T',
  p = 'NO', q = 'N',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=49.500, b=0.042000}}
}

mechanism[14] = {
  type = 'V-T',
  p = 'NO', q = 'O',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=49.500, b=0.042000}}
}

mechanism[15] = {
  type = 'V-T',
  p = 'NO', q = 'NO',
  mode_p = 0,
  rate = 'Landau-Teller',
  relaxation_time = {model='ParkHTC2', sigma=1.0000e-21, submodel={model='Millikan-White', a=49.500, b=0.042000}}
}

mechanism[16] = {
  type = 'C-V',
  p = 'N2',
  rate = 'Marrone-Treanor',
  mode_p = 0,
  reaction_index = 0,
  coupling_model = {model='MarroneTreanorDissociation', D=945360.000000, Thetav=3393.440000, U=37900.054122}
}

mechanism[17] = {
  type = 'C-V',
  p = 'O2',
  rate = 'Marrone-Treanor',
  mode_p = 0,
  reaction_index = 1,
  coupling_model = {model='ModifiedMarroneTreanorDissociation', T_D=59937.459378, Thetav=2273.540000, Ustar=40000.000000, aU=0.150000, non_boltzmann=0.100000}
}

mechanism[18] = {
  type = 'C-V',
  p = 'NO',
  rate = 'Marrone-Treanor',
  mode_p = 0,
  reaction_index = 2,
  coupling_model = {model='ImpartialDissociation', D=630583.693000, Thetav=2739.700000}
}

