rate = { A = 1.92e11,
         n = -0.5,
         C = 1.131e5,
         rctIndex = -1}

